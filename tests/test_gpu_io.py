"""State files (vpm_save / vpm_load, the role of vpm.save / vpm.read!): a
saved and reloaded field is the same field, bit for bit, including static
particles, SFS memory, volumes and circulations, and steps identically
afterwards.  Version-1 files (no vol / circulation) still load; files whose
static flags disagree with their header are rejected."""
import ctypes
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300 import vpm
from flowunsteady_gb300.workloads import leapfrog_rings, uniform_box
from tests.helpers import Ctx, scheme

pytestmark = pytest.mark.gpu


def test_save_load_round_trip_and_identical_continuation(tmp_path):
    X, G, S = leapfrog_rings(nstations=40)
    Xs, Gs, Ss = uniform_box(50, seed_index=150)
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    sc = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    n = X.shape[0] + 50
    with Ctx(n) as a, Ctx(n) as b:
        a.set(X, G, S)
        a.append(Xs, Gs * 0, Ss, static=True)
        a.step(sc, 0.005, nsteps=3)
        prefix = str(tmp_path / "rings")
        a.rc(a.lib.vpm_save(a.p, prefix.encode(), 3))
        xmf = tmp_path / "rings.pfield.3.xmf"
        root = ET.parse(xmf).getroot()
        items = root.findall(".//DataItem")
        assert [it.get("Dimensions") for it in items] == [f"{n} 3", f"{n} 3", f"{n}", f"{n} 3",
                                                          f"{n}", f"{n}", f"{n}"]
        assert (tmp_path / "rings.pfield.3.bin").stat().st_size == 64 + 104 * n
        b.rc(b.lib.vpm_load(b.p, str(tmp_path / "rings.pfield.3.bin").encode(), 1))
        na, nsa, nb, nsb = (ctypes.c_int64() for _ in range(4))
        a.rc(a.lib.vpm_get_np(a.p, ctypes.byref(na), ctypes.byref(nsa)))
        b.rc(b.lib.vpm_get_np(b.p, ctypes.byref(nb), ctypes.byref(nsb)))
        assert (na.value, nsa.value) == (nb.value, nsb.value) == (n, 50)
        t, nt = ctypes.c_double(), ctypes.c_int64()
        b.rc(b.lib.vpm_get_time(b.p, ctypes.byref(t), ctypes.byref(nt)))
        assert nt.value == 3 and abs(t.value - 0.015) < 1e-15
        for u, v in zip(a.state(), b.state()):
            assert np.array_equal(u, v)
        assert np.array_equal(a.sfs()[0], b.sfs()[0])
        a.step(sc, 0.005, nsteps=2)
        b.step(sc, 0.005, nsteps=2)
        for u, v in zip(a.state(), b.state()):
            assert np.array_equal(u, v)


def test_python_save_read_and_bad_files(tmp_path):
    X, G, S = uniform_box(300, seed_index=151)
    pf = vpm.ParticleField(400)
    pf.set_particles(X, G, S)
    xmf = vpm.save(pf, "box", path=str(tmp_path), num=7)
    assert xmf.endswith("box.pfield.7.xmf")
    pf2 = vpm.ParticleField(400)
    vpm.read(pf2, xmf)
    for u, v in zip(pf.state(), pf2.state()):
        assert np.array_equal(u, v)
    bad = tmp_path / "junk.bin"
    bad.write_bytes(b"not a field" * 10)
    with pytest.raises(L.VPMError):
        vpm.read(pf2, str(bad))
    small = vpm.ParticleField(100)
    with pytest.raises(L.VPMError):
        vpm.read(small, xmf)


def _write_v1(path, X, G, S, C, st, n_static, t=0.25, nt=5):
    """A version-1 state file: header, X, Γ, σ, C, static flag (FP64)."""
    import struct
    n = X.shape[0]
    head = b"VPMFIELD" + struct.pack("<IIqqdq", 1, 64, n, n_static, t, nt) + bytes(16)
    assert len(head) == 64
    with open(path, "wb") as f:
        f.write(head)
        for a in (X, G, S, C, st):
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def test_version1_files_load_and_bad_static_flags_are_rejected(tmp_path):
    X, G, S = uniform_box(120, seed_index=152)
    C = np.random.default_rng(1).uniform(0, 0.3, (120, 3))
    st = np.zeros(120)
    st[-20:] = 1.0
    good = tmp_path / "v1.bin"
    _write_v1(good, X, G, S, C, st, 20)
    with Ctx(150) as c:
        c.rc(c.lib.vpm_load(c.p, str(good).encode(), 1))
        Xg, Gg, Sg = c.state()
        assert np.array_equal(Xg, X) and np.array_equal(Gg, G) and np.array_equal(Sg, S)
        assert np.array_equal(c.sfs()[0], C)
        vol, circ = np.empty(120), np.empty(120)
        flags = (ctypes.c_int32 * 120)()
        c.rc(c.lib.vpm_get_attributes(c.p, 0, 120, L.dptr(vol), 1, L.dptr(circ), 1, flags))
        assert np.all(vol == 0.0) and np.all(circ == 1.0)
        assert list(flags) == [0] * 100 + [1] * 20
        # Flags that disagree with the static count, or that are not 0/1.
        for bad_st, ns in ((np.r_[np.ones(20), np.zeros(100)], 20), (st, 19), (st * 0.5, 20)):
            bad = tmp_path / "bad.bin"
            _write_v1(bad, X, G, S, C, bad_st, ns)
            assert c.lib.vpm_load(c.p, str(bad).encode(), 0) == L.ERR_INVALID


def test_attributes_and_mixed_static_flags_survive_a_round_trip(tmp_path):
    X, G, S = uniform_box(90, seed_index=153)
    rng = np.random.default_rng(2)
    vol, circ = rng.uniform(0, 1e-3, 90), rng.uniform(0.5, 2.0, 90)
    with Ctx(100) as a, Ctx(100) as b:
        a.set(X[:40], G[:40], S[:40])
        a.append(X[40:60], G[40:60], S[40:60], static=True)
        a.append(X[60:], G[60:], S[60:])            # free particles after static ones
        a.rc(a.lib.vpm_set_attributes(a.p, 0, 90, L.dptr(vol), 1, L.dptr(circ), 1, None, 3))
        prefix = str(tmp_path / "mixed")
        a.rc(a.lib.vpm_save(a.p, prefix.encode(), -1))
        b.rc(b.lib.vpm_load(b.p, (prefix + ".pfield.bin").encode(), 0))
        v2, c2 = np.empty(90), np.empty(90)
        fl = (ctypes.c_int32 * 90)()
        b.rc(b.lib.vpm_get_attributes(b.p, 0, 90, L.dptr(v2), 1, L.dptr(c2), 1, fl))
        assert np.array_equal(v2, vol) and np.array_equal(c2, circ)
        assert list(fl) == [0] * 40 + [1] * 20 + [0] * 30
        for u, w in zip(a.state(), b.state()):
            assert np.array_equal(u, w)
