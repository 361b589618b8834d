"""pic_energy_noalloc: the energy/momentum sums for caller-owned device
arrays, computed without any device allocation (for callers that cannot
allocate: inside stream capture, under a fixed memory pool, or with their own
allocator).  Checked against pic_energy on the same state, two calls in a
row, through the C ABI.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from picpp_gb300 import initstate as I

pytestmark = pytest.mark.gpu


def test_energy_noalloc_matches_pic_energy_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import picpp_gb300 as P
    L = P.load_library()
    st = I.buneman_plasma(16, 8, 8, ppc=3, seed=71)
    rng = np.random.default_rng(72)
    st.E = st.E + 0.05 * rng.standard_normal(st.E.shape)
    st.B = st.B + 0.05 * rng.standard_normal(st.B.shape)
    sim = P.GpuSimulation(st.box, P.BUNEMAN, particle_real=P.F64, sort_every=0)
    sim.upload_state(st)
    ref = sim.updateEnergy()

    # the caller's own device buffers (allocated here by the test, not by the library)
    dev = torch.device("cuda:0")
    E = torch.from_numpy(np.ascontiguousarray(st.E.reshape(-1))).to(dev)
    B = torch.from_numpy(np.ascontiguousarray(st.B.reshape(-1))).to(dev)
    moms = [[torch.from_numpy(np.ascontiguousarray(sp[k])).to(dev) for k in ("px", "py", "pz")] for sp in st.species]
    ns = len(st.species)
    counts = (C.c_long * ns)(*[len(sp["cell"]) for sp in st.species])
    masses = (C.c_double * ns)(*[sp["m"] for sp in st.species])
    weights = (C.c_double * ns)(*[sp["w"] for sp in st.species])
    px = (C.c_void_p * ns)(*[m[0].data_ptr() for m in moms])
    py = (C.c_void_p * ns)(*[m[1].data_ptr() for m in moms])
    pz = (C.c_void_p * ns)(*[m[2].data_ptr() for m in moms])
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    for _ in range(2):
        out = np.zeros(6)
        st_code = L.pic_energy_noalloc(st.box.nx, st.box.ny, st.box.nz, st.box.dx, st.box.dy, st.box.dz,
                                       E.data_ptr(), B.data_ptr(), ns, counts, masses, weights, px, py, pz,
                                       stream, out.ctypes.data_as(C.POINTER(C.c_double)))
        assert st_code == P.PIC_OK
        assert np.allclose(out, ref, rtol=1e-12, atol=1e-14)

    # more species than the static scratch holds is refused
    too_many = P.PIC_NOALLOC_MAX_SPECIES + 1 if hasattr(P, "PIC_NOALLOC_MAX_SPECIES") else 17
    big = (C.c_long * too_many)()
    out = np.zeros(6)
    st_code = L.pic_energy_noalloc(st.box.nx, st.box.ny, st.box.nz, st.box.dx, st.box.dy, st.box.dz,
                                   E.data_ptr(), B.data_ptr(), too_many, big, None, None, None, None, None,
                                   stream, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert st_code == 1
    sim.close()
