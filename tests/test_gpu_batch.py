"""Batched fields: one persistent launch over a flattened work queue per pair
pass, checked against separate per-field contexts (FP64) and the oracle."""
import numpy as np
import pytest

from flowunsteady_gb300 import _lib as L
from flowunsteady_gb300.batch import FieldBatch
from flowunsteady_gb300.workloads import uniform_box
from tests.helpers import Ctx, rel_l2, rel_max, scheme

pytestmark = pytest.mark.gpu
SIZES = [37, 2048, 700, 5000, 1, 129]


def fields():
    out = []
    for f, n in enumerate(SIZES):
        X, G, S = uniform_box(n, seed_index=100 + f)
        out.append((X, G * 100, S * 2))
    return out


def test_batch_uj_matches_separate_fields(oracle):
    fs = fields()
    b = FieldBatch(SIZES)
    for f, (X, G, S) in enumerate(fs):
        b.set_field(f, X, G, S)
    for prec, tol in ((L.PREC_FP64, 1e-12), (L.PREC_FP32C, 1e-5)):
        b.eval_UJ(L.KERNEL_GAUSSIANERF, prec)
        for f, (X, G, S) in enumerate(fs):
            U, J = b.get_UJ(f)
            U0, J0 = oracle.uj_direct(1, X, G, S)
            if X.shape[0] == 1:
                assert np.all(U == 0)
                continue
            assert rel_l2(U, U0) <= tol and rel_l2(J, J0) <= tol
    b.close()


def test_batch_step_matches_separate_contexts():
    fs = fields()
    sc = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, nu=1e-4, rlxf=0.5)
    b = FieldBatch(SIZES)
    for f, (X, G, S) in enumerate(fs):
        b.set_field(f, X, G, S)
    b.step(0.005, sc, nsteps=3)
    for f, (X, G, S) in enumerate(fs):
        with Ctx(X.shape[0]) as c:
            c.set(X, G, S)
            c.step(sc, 0.005, nsteps=3)
            ref = c.state()
        got = b.get_field(f)
        for a, r in zip(got, ref):
            assert rel_max(a, r) <= 1e-10
    b.close()


def test_batch_fp32c_step_in_morton_order():
    # FP32 batch passes run each field along the Morton curve of its own cube
    # (gathers of x, Γ, σ, v, w; scatters of U, J, DJ and the ζ sums).  Three
    # steps with the analytic dynamic SFS against separate FP64 contexts.
    fs = fields()
    flags = L.SFS_CLIP_BACKSCATTER | L.SFS_FORCE_POSITIVE | L.SFS_ANALYTIC_DSIGMA
    sc = scheme(kernel=1, prec=L.PREC_FP32C, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    b = FieldBatch(SIZES)
    for f, (X, G, S) in enumerate(fs):
        b.set_field(f, X, G, S)
    b.step(0.005, sc, nsteps=3)
    sc64 = scheme(kernel=1, prec=L.PREC_FP64, sfs=L.SFS_DYNAMIC, flags=flags, nu=1e-4)
    err = []
    for f, (X, G, S) in enumerate(fs):
        with Ctx(X.shape[0]) as c:
            c.set(X, G, S)
            c.step(sc64, 0.005, nsteps=3)
            ref = c.state()
        got = b.get_field(f)
        err.append((float(np.abs(got[0] - ref[0]).max()), rel_l2(got[1], ref[1]),
                    rel_max(got[2], ref[2])))
    b.close()
    for dx, dg, ds in err:
        assert dx <= 1e-7 and dg <= 2e-6 and ds <= 5e-7, err


def test_batch_particle_order_changes_only_the_summation_order():
    fs = fields()
    res = {}
    for mode in (L.ORDER_AUTO, L.ORDER_CALLER):
        b = FieldBatch(SIZES)
        b.set_particle_order(mode)
        for f, (X, G, S) in enumerate(fs):
            b.set_field(f, X, G, S)
        b.eval_UJ(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
        res[mode] = [b.get_UJ(f) for f in range(len(SIZES))]
        b.close()
    for f in range(len(SIZES)):
        if SIZES[f] == 1:
            continue
        (Ua, Ja), (Uc, Jc) = res[L.ORDER_AUTO][f], res[L.ORDER_CALLER][f]
        assert rel_l2(Ua, Uc) <= 1e-6 and rel_l2(Ja, Jc) <= 1e-6, f


def test_batch_fields_of_different_shapes_run_as_separate_launches(oracle):
    # A field of 200,000 particles takes the 128x4 shape (the default from
    # 196,608 particles on), the small ones 128x2 (or what the per-device table
    # holds for their size bucket): one persistent launch per shape.  Every
    # field still matches the oracle.
    sizes = [3000, 200000, 5000, 700]
    fs = []
    for f, n in enumerate(sizes):
        X, G, S = uniform_box(n, seed_index=110 + f)
        fs.append((X, G * 100, S * 2))
    b = FieldBatch(sizes)
    for f, (X, G, S) in enumerate(fs):
        b.set_field(f, X, G, S)
    b.eval_UJ(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    shapes = b.shapes()
    assert shapes[1] == (128, 4) and len(set(shapes)) >= 2
    rng = np.random.default_rng(111)
    for f, (X, G, S) in enumerate(fs):
        U, J = b.get_UJ(f)
        idx = rng.choice(X.shape[0], min(400, X.shape[0]), replace=False)
        U0, J0 = oracle.uj_direct(1, X, G, S, Xt=X[idx])
        assert rel_l2(U[idx], U0) <= 1e-5 and rel_l2(J[idx], J0) <= 1e-5, f
    b.close()


def test_batch_autotune_per_size_bucket(oracle):
    sizes = [2048, 2500, 9000, 12000, 40000]
    fs = []
    for f, n in enumerate(sizes):
        X, G, S = uniform_box(n, seed_index=120 + f)
        fs.append((X, G * 100, S * 2))
    b = FieldBatch(sizes)
    for f, (X, G, S) in enumerate(fs):
        b.set_field(f, X, G, S)
    ms = b.autotune(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    assert ms > 0
    shapes = b.shapes()
    assert all(s in {(128, 2), (128, 4), (256, 2)} for s in shapes)
    assert shapes[0] == shapes[1] and shapes[2] == shapes[3]   # same size bucket, same shape
    b.eval_UJ(L.KERNEL_GAUSSIANERF, L.PREC_FP32C)
    for f, (X, G, S) in enumerate(fs):
        U, J = b.get_UJ(f)
        idx = np.random.default_rng(f).choice(X.shape[0], 300, replace=False)
        U0, J0 = oracle.uj_direct(1, X, G, S, Xt=X[idx])
        assert rel_l2(U[idx], U0) <= 1e-5 and rel_l2(J[idx], J0) <= 1e-5, f
    b.close()
