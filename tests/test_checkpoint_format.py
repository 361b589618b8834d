"""The host-side reader and writer of the binary checkpoint
(picpp_gb300.checkpoint): round trips, layout and rejected files.  No GPU."""
import numpy as np
import pytest

from picpp_gb300 import checkpoint as K
from picpp_gb300 import initstate as I


def _equal_states(a, b):
    assert a.box == b.box
    assert np.array_equal(a.E, b.E) and np.array_equal(a.B, b.B)
    for sa, sb in zip(a.species, b.species):
        for k in ("q", "m", "w"):
            assert sa[k] == sb[k]
        for k in ("cell", "ox", "oy", "oz", "px", "py", "pz"):
            assert np.array_equal(sa[k], sb[k]), k


def test_header_is_120_bytes():
    assert K.HEADER.size == 120


@pytest.mark.parametrize("solver,real", [(0, 1), (1, 1), (1, 0)])
def test_state_round_trip(tmp_path, solver, real):
    st = I.beams_plasma(6, 5, 4, ppc=2, seed=5) if solver else I.buneman_plasma(6, 5, 4, ppc=2, seed=5)
    ck = K.from_state(st, solver, real, step=7)
    p = tmp_path / "s.ckpt"
    K.write(p, ck)
    back = K.read(p)
    assert back.solver == solver and back.particle_real == real and back.step == 7 and not back.sorted
    assert back.params is None
    n = back.box.nx * back.box.ny * back.box.nz
    size = 120 + sum(24 + 8 + len(s["cell"]) * (8 + 6 * (8 if real else 4)) for s in st.species)
    size += 2 * 3 * n * (8 if (real or solver) else 4) + 3 * n * 8
    assert p.stat().st_size == size
    got = K.to_state(back)
    if real:
        _equal_states(got, st)
    else:
        for sa, sb in zip(got.species, st.species):
            for k in ("ox", "px"):
                assert np.array_equal(sa[k], sb[k].astype(np.float32).astype(np.float64))


def test_sorted_offsets_ids_and_network_round_trip(tmp_path):
    st = I.buneman_plasma(4, 4, 2, ppc=3, seed=6)
    ck = K.from_state(st, 0, 1)
    rng = np.random.default_rng(1)
    for sp in ck.species:
        sp["id"] = rng.permutation(len(sp["cell"])).astype(np.int32)
        sp["off"] = np.arange(33, dtype=np.int32)
    ck.sorted = True
    ck.params = rng.standard_normal(101).astype(np.float32)
    ck.J = rng.standard_normal((3, 2, 4, 4))
    K.write(tmp_path / "a.ckpt", ck)
    back = K.read(tmp_path / "a.ckpt")
    assert back.sorted
    assert np.array_equal(back.params, ck.params)
    assert np.array_equal(back.J, ck.J)
    for a, b in zip(back.species, ck.species):
        assert np.array_equal(a["id"], b["id"]) and np.array_equal(a["off"], b["off"])
    # to_state puts every species back in id order
    s0 = K.to_state(back).species[0]
    o = np.argsort(ck.species[0]["id"])
    assert np.array_equal(s0["px"], ck.species[0]["px"][o])


def test_rejects_foreign_and_truncated_files(tmp_path):
    st = I.buneman_plasma(4, 4, 2, ppc=1, seed=7)
    p = tmp_path / "c.ckpt"
    K.write(p, K.from_state(st, 0, 1))
    raw = p.read_bytes()
    (tmp_path / "t.ckpt").write_bytes(raw[:-8])
    with pytest.raises(ValueError):
        K.read(tmp_path / "t.ckpt")
    (tmp_path / "m.ckpt").write_bytes(b"NOTAPIC!" + raw[8:])
    with pytest.raises(ValueError):
        K.read(tmp_path / "m.ckpt")
    (tmp_path / "x.ckpt").write_bytes(raw + b"\0" * 3)
    with pytest.raises(ValueError):
        K.read(tmp_path / "x.ckpt")
