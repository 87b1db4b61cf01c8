"""Discrete adjoint (shm_forward_backward) against finite differences, the FP64
oracle and itself (checkpoint interval, precision, batching)."""
import numpy as np
import pytest

from oracle.oracle import OracleProblem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def adjoint_case(pkg, nex=6, ney=5, nft=260, seed=0):
    """Plate with a hidden damage map; the model starts undamaged."""
    scs, run = pkg.workloads.plate_force(nex=nex, ney=ney, L=0.006 * max(nex, ney), T=1e-4, f=300e3, n_out=4,
                                         radius=0.01)
    run.nft = nft
    sc = scs[0]
    sc.signal = sc.signal[:nft]
    fen = nex * ney
    rng = np.random.default_rng(seed)
    keep_true = np.ones(fen)
    keep_true[rng.choice(fen, 4, replace=False)] = 0.5
    sc.elem_keep = keep_true
    plan = pkg.Plan([sc], run, precision=64, path=1)
    target = plan.forward()[0]["displ"]
    plan.close()
    sc.elem_keep = np.ones(fen) * 0.9 + 0.1 * rng.random(fen)  # current model
    return sc, run, target


def misfit_gpu(pkg, sc, run, target, keep, prec=64):
    sc2 = pkg.Scenario(**{**sc.__dict__, "elem_keep": keep})
    p = pkg.Plan([sc2], run, precision=prec, path=1)
    d = p.forward()[0]["displ"]
    p.close()
    r = (d - target)[run.nn_first - 1:]
    return 0.5 * np.sum(r * r)


def test_adjoint_gradient_matches_finite_differences(pkg):
    sc, run, target = adjoint_case(pkg)
    plan = pkg.Plan([sc], run, precision=64, path=1)
    mis, grad = plan.forward_backward([target], ckpt_every=40)
    plan.close()
    g = grad[0]
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    assert abs(mis[0] - misfit_gpu(pkg, sc, run, target, sc.elem_keep)) <= 1e-12 * mis[0]
    rng = np.random.default_rng(1)
    idx = rng.choice(len(g), 8, replace=False)
    eps = 1e-4
    for e in idx:
        kp = sc.elem_keep.copy()
        km = sc.elem_keep.copy()
        kp[e] -= eps  # d_e + eps
        km[e] += eps
        fd = (misfit_gpu(pkg, sc, run, target, kp) - misfit_gpu(pkg, sc, run, target, km)) / (2 * eps)
        assert abs(fd - g[e]) <= 1e-5 * np.abs(g).max(), (e, fd, g[e])


def test_adjoint_gradient_matches_oracle_finite_differences(pkg):
    """Central differences of the FP64 oracle's misfit (the reference loop
    restated) pin the GPU gradient."""
    sc, run, target = adjoint_case(pkg, nex=4, ney=4, nft=200, seed=3)
    plan = pkg.Plan([sc], run, precision=64, path=1)
    _, grad = plan.forward_backward([target], ckpt_every=50)
    plan.close()
    g = grad[0]

    def orc_misfit(keep):
        orc = OracleProblem(sc.mesh["nodes"], sc.mesh["coords"], sc.mat_table, None, keep)
        d = orc.run(run.dt, run.nft, sc.signal, nn_first=run.nn_first, eta_xy=run.eta_xy, eta_z=run.eta_z,
                    force_dof=sc.force_dof, force_val=sc.force_val, out_dof=sc.out_dof, h=run.h)["displ"]
        r = (d - target)[run.nn_first - 1:]
        return 0.5 * np.sum(r * r)

    eps = 1e-4
    for e in (0, 5, 9, 15):
        kp = sc.elem_keep.copy()
        km = sc.elem_keep.copy()
        kp[e] -= eps
        km[e] += eps
        fd = (orc_misfit(kp) - orc_misfit(km)) / (2 * eps)
        assert abs(fd - g[e]) <= 1e-5 * np.abs(g).max(), (e, fd, g[e])


def test_adjoint_checkpoint_interval_and_precision(pkg):
    sc, run, target = adjoint_case(pkg, seed=2)
    res = {}
    for prec, k in ((64, 260), (64, 7), (32, 33)):
        plan = pkg.Plan([sc], run, precision=prec, path=1)
        res[(prec, k)] = plan.forward_backward([target], ckpt_every=k)
        plan.close()
    g64a, g64b, g32 = res[(64, 260)][1][0], res[(64, 7)][1][0], res[(32, 33)][1][0]
    assert rel(g64b, g64a) <= 1e-12
    assert rel(g32, g64a) <= 1e-3
    assert abs(res[(32, 33)][0][0] - res[(64, 260)][0][0]) <= 1e-3 * res[(64, 260)][0][0]


def test_adjoint_batch_equals_solo(pkg):
    cases = [adjoint_case(pkg, seed=s) for s in range(3)]
    run = cases[0][1]
    scs = [c[0] for c in cases]
    plan = pkg.Plan(scs, run, precision=32, path=1)
    mis, grads = plan.forward_backward([c[2] for c in cases], ckpt_every=50)
    plan.close()
    for s, (sc, _, tgt) in enumerate(cases):
        p1 = pkg.Plan([sc], run, precision=32, path=1)
        m1, g1 = p1.forward_backward([tgt], ckpt_every=50)
        p1.close()
        np.testing.assert_array_equal(grads[s], g1[0])
        assert mis[s] == m1[0]


@pytest.mark.parametrize("prec", [64, 32])
def test_adjoint_on_structured_plan(pkg, prec):
    """A plan on the structured fused kernels runs its forward pass and the
    segment recomputes on those kernels (recompute bit-identical to the
    forward pass); the gradient matches the general-path plan's."""
    sc, run, target = adjoint_case(pkg, seed=4)
    res = {}
    for path in (1, 2):
        plan = pkg.Plan([sc], run, precision=prec, path=path)
        assert plan.info["path"] == path
        plan.set_adjoint_store(0)  # recompute every segment
        res[path] = plan.forward_backward([target], ckpt_every=37)
        assert plan.stored_segments() == 0
        t = plan.forward_backward_timing()
        assert t["forward_ms"] > 0 and t["recompute_ms"] > 0 and t["adjoint_ms"] > 0
        plan.close()
    tol = 1e-10 if prec == 64 else 1e-4
    assert rel(res[2][1][0], res[1][1][0]) <= tol
    assert abs(res[2][0][0] - res[1][0][0]) <= tol * res[1][0][0]


@pytest.mark.parametrize("path", [1, 2])
def test_adjoint_stored_segments_equal_recompute(pkg, path):
    """Keeping the last segments' forward states instead of recomputing them
    changes nothing: the states are the same bits."""
    sc, run, target = adjoint_case(pkg, seed=5)
    plan = pkg.Plan([sc], run, precision=32, path=path)
    k = 30
    nck = -(-(run.nft - run.nn_first + 1) // k)
    state_bytes = 4 * 5 * plan.info["nnode"]
    got = {}
    for name, cap in (("none", 0), ("part", (nck // 2) * k * state_bytes), ("all", None)):
        plan.set_adjoint_store(cap)
        got[name] = plan.forward_backward([target], ckpt_every=k)
        got[name + "_n"] = plan.stored_segments()
    plan.close()
    assert got["none_n"] == 0 and 0 < got["part_n"] < nck and got["all_n"] == nck
    for name in ("part", "all"):
        np.testing.assert_array_equal(got[name][1][0], got["none"][1][0])
        assert got[name][0][0] == got["none"][0][0]


def test_adjoint_with_persistent_forward(pkg):
    """A plan that steps persistently runs the forward pass of
    forward_backward in the persistent kernel (the recompute and the adjoint
    sweep keep their per-step launches): the states are the same bits, so
    misfit and gradient equal those of the per-step plan exactly, with part of
    the segments stored and the rest recomputed."""
    sc, run, target = adjoint_case(pkg, seed=6)
    got = {}
    for persistent in (False, True):
        plan = pkg.Plan([sc], run, precision=32, path=2)
        if persistent:
            plan.set_persistent(True)
        k = 30
        nck = -(-(run.nft - run.nn_first + 1) // k)
        plan.set_adjoint_store((nck // 2) * k * 4 * 5 * plan.info["nnode"])
        got[persistent] = plan.forward_backward([target], ckpt_every=k)
        assert 0 < plan.stored_segments() < nck
        plan.close()
    np.testing.assert_array_equal(got[True][1][0], got[False][1][0])
    assert got[True][0][0] == got[False][0][0]
