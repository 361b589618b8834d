"""pic_energy_noalloc: the energy/momentum sums for caller-owned device
arrays, computed without any device allocation, for callers that cannot
allocate device memory where they need the sums (a memory pool fixed at
start-up, an allocator of their own).  Checked against pic_energy on the same
state, two calls in a row, through the C ABI; against a NumPy sum for species
of very different sizes, an empty species and no B grid; and the device's
free memory is unchanged by repeated calls.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from picpp_gb300 import initstate as I

pytestmark = pytest.mark.gpu


def _lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import picpp_gb300 as P
    return P, P.load_library()


def _call(L, box, E, B, species, stream):
    """species: list of (m, w, px, py, pz) with torch device tensors (or None for an empty one)."""
    ns = len(species)
    counts = (C.c_long * max(ns, 1))(*[0 if s[2] is None else s[2].numel() for s in species])
    masses = (C.c_double * max(ns, 1))(*[s[0] for s in species])
    weights = (C.c_double * max(ns, 1))(*[s[1] for s in species])
    ptr = [(C.c_void_p * max(ns, 1))(*[None if s[2 + a] is None else s[2 + a].data_ptr() for s in species])
           for a in range(3)]
    out = np.zeros(6)
    code = L.pic_energy_noalloc(box[0], box[1], box[2], box[3], box[4], box[5],
                                None if E is None else E.data_ptr(), None if B is None else B.data_ptr(),
                                ns, counts, masses, weights, ptr[0], ptr[1], ptr[2], stream,
                                out.ctypes.data_as(C.POINTER(C.c_double)))
    return code, out


def test_energy_noalloc_matches_pic_energy_twice():
    P, L = _lib()
    import torch
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
    sp = [(s["m"], s["w"]) + tuple(torch.from_numpy(np.ascontiguousarray(s[k])).to(dev) for k in ("px", "py", "pz"))
          for s in st.species]
    box = (st.box.nx, st.box.ny, st.box.nz, st.box.dx, st.box.dy, st.box.dz)
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    for _ in range(2):
        code, out = _call(L, box, E, B, sp, stream)
        assert code == P.PIC_OK
        assert np.allclose(out, ref, rtol=1e-12, atol=1e-14)

    # more species than the static scratch holds is refused
    too_many = P.PIC_NOALLOC_MAX_SPECIES + 1
    big = (C.c_long * too_many)()
    out = np.zeros(6)
    code = L.pic_energy_noalloc(*box, E.data_ptr(), B.data_ptr(), too_many, big, None, None, None, None, None,
                                stream, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert code == P.PIC_ERR_ARG
    sim.close()


def _numpy_sums(box, E, B, species):
    kin, mom = 0.0, np.zeros(3)
    for m, w, px, py, pz in species:
        if px is None:
            continue
        gam = np.sqrt((px * px + py * py + pz * pz) / (m * m) + 1.0)
        kin += np.sum((gam - 1.0) * m * w)
        mom += w * np.array([px.sum(), py.sum(), pz.sum()])
    scale = box[3] * box[4] * box[5] / (8 * np.pi)
    e = 0.0 if E is None else np.sum(E * E) * scale
    b = 0.0 if B is None else np.sum(B * B) * scale
    return np.array([kin, e, b, mom[0], mom[1], mom[2]])


def test_energy_noalloc_uneven_species_and_no_b_grid_allocate_nothing():
    """Species of 10 and 50,000 particles (different reduction widths), an
    empty species between them, no B grid; repeated calls leave the device's
    free memory unchanged."""
    P, L = _lib()
    import torch
    rng = np.random.default_rng(90)
    box = (12, 10, 6, 0.3, 0.2, 0.25)
    N = box[0] * box[1] * box[2]
    E = rng.standard_normal(3 * N)
    host = [(1.0, 0.7) + tuple(rng.standard_normal(10) for _ in range(3)),
            (3.0, 1.1, None, None, None),
            (100.0, 0.02) + tuple(5.0 * rng.standard_normal(50000) for _ in range(3))]
    ref = _numpy_sums(box, E, None, host)
    dev = torch.device("cuda:0")
    Ed = torch.from_numpy(E).to(dev)
    sp = [(m, w) + ((None,) * 3 if px is None else tuple(torch.from_numpy(a).to(dev) for a in (px, py, pz)))
          for m, w, px, py, pz in host]
    stream = torch.cuda.current_stream().cuda_stream
    torch.cuda.synchronize()
    code, out = _call(L, box, Ed, None, sp, stream)       # first call: symbol lookup, module load
    assert code == P.PIC_OK
    assert np.allclose(out, ref, rtol=1e-11, atol=1e-12), (out, ref)
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        code, out2 = _call(L, box, Ed, None, sp, stream)
        assert code == P.PIC_OK
        assert np.array_equal(out2, out)                 # fixed-order sums: the same bits every call
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
