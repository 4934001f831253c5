"""State files (vpm_save / vpm_load, the role of vpm.save / vpm.read!): a
saved and reloaded field is the same field, bit for bit, including static
particles and SFS memory, and steps identically afterwards."""
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
        assert [it.get("Dimensions") for it in items] == [f"{n} 3", f"{n} 3", f"{n}", f"{n} 3", f"{n}"]
        assert (tmp_path / "rings.pfield.3.bin").stat().st_size == 64 + 88 * n
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
