"""Persistent stepping of FP32 structured plans (shm_set_persistent): all
steps of a call in one cooperative launch whose CTAs meet at a device-wide
barrier between steps.  It must give the same bits as one launch per step,
also when the grid is smaller than the task list (each CTA then takes several
task groups per step), and a barrier wait that runs out must come back as
SHM_ERR_TIMEOUT with the plan still usable.  The timeout is made by a zero
poll limit: the CTAs that are not last at the first barrier give up at once
(no device fault, no endless wait)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def batch(pkg, n, seed, nmin, nmax, nft, sensors=False):
    scs = [pkg.workloads.random_plate(np.random.default_rng([seed, s]), edge=6.25e-3, nmin=nmin, nmax=nmax)
           for s in range(n)]
    dt = 7e-8
    for sc in scs:
        _, sc.signal = pkg.hanning_signal(dt, nft, sc.carrier / 5, sc.carrier)
        if sensors:
            sc.sensors = [np.array([5, 6, 7], np.int32)]
            sc.pzt = dict(pzt_thickness=0.2e-3, g33=1.5e-8, e31=-5.4, e32=-5.4)
    return scs, pkg.RunConfig(dt=dt, nft=nft, eta_xy=4e2, eta_z=4e3, h=3.9e-3, frm_int=100 if sensors else 0)


def run_both(pkg, scs, run, **kw):
    out = []
    for persistent in (False, True):
        plan = pkg.Plan(scs, run, precision=32, path=2, steps_per_graph=50, **kw)
        if persistent:
            plan.set_persistent(True)
            assert plan.info["persistent"] and plan.info["launches_per_step"] == 0
        res = plan.forward(want_frames=run.frm_int > 0)
        U, Uo = plan.get_state()
        plan.close()
        out.append((res, U, Uo))
    return out


@pytest.mark.parametrize("tile", [16, 32])
def test_persistent_equals_per_step_launches(pkg, tile):
    """Random plates with damage zones, PZT sensors and frames: displacement,
    voltage, frames and the final state bit for bit."""
    scs, run = batch(pkg, 3, 11, 20, 45, 400, sensors=True)
    (ra, Ua, Uoa), (rb, Ub, Uob) = run_both(pkg, scs, run, tile_elems=tile, rows_per_block=8)
    for a, b in zip(ra, rb):
        for key in ("displ", "voltage", "frames"):
            np.testing.assert_array_equal(a[key], b[key])
        assert np.abs(a["displ"]).max() > 0
    np.testing.assert_array_equal(Ua, Ub)
    np.testing.assert_array_equal(Uoa, Uob)


def test_persistent_grid_smaller_than_task_list(pkg):
    """One element row per task over 48 plates: far more task groups than
    co-resident CTAs, so every CTA loops over several groups per step."""
    scs, run = batch(pkg, 48, 12, 25, 45, 200)
    # one task per element row and strip: at least 48 x 25, against at most
    # two resident CTAs per multiprocessor
    ntask = sum((len(np.unique(np.round(np.asarray(sc.mesh["coords"])[:, 1], 9))) - 1) // 5 for sc in scs)
    assert ntask >= 48 * 25
    (ra, Ua, _), (rb, Ub, _) = run_both(pkg, scs, run, tile_elems=32, rows_per_block=1)
    for a, b in zip(ra, rb):
        np.testing.assert_array_equal(a["displ"], b["displ"])
    np.testing.assert_array_equal(Ua, Ub)


def test_persistent_barrier_timeout_is_reported(pkg):
    scs, run = pkg.workloads.plate_force(nex=20, ney=20, L=0.25, T=4e-5)
    run.nft = min(run.nft, 300)
    scs[0].signal = scs[0].signal[:run.nft]
    plan = pkg.Plan(scs, run, precision=32, path=2, tile_elems=32, rows_per_block=1)
    ref = plan.forward()[0]
    plan.set_persistent(True, spin_limit=0)
    with pytest.raises(pkg.native.ShmError) as ei:
        plan.forward()
    assert ei.value.status == pkg.native.SHM_ERR_TIMEOUT
    # the context and the plan stay usable: default limit, same bits as the
    # per-step launches
    plan.set_persistent(True)
    again = plan.forward()[0]
    plan.close()
    np.testing.assert_array_equal(again["displ"], ref["displ"])


def test_persistent_needs_an_fp32_structured_plan(pkg):
    scs, run = pkg.workloads.plate_force(nex=6, ney=6, L=0.075, T=1e-5)
    for prec, path in ((64, 2), (32, 1)):
        plan = pkg.Plan(scs, run, precision=prec, path=path)
        with pytest.raises(pkg.native.ShmError) as ei:
            plan.set_persistent(True)
        assert ei.value.status == pkg.native.SHM_ERR_BAD_ARG
        plan.set_persistent(False)
        plan.close()


def test_persistent_with_pressure_loading(pkg):
    """Pressure loading (interpolated nodal frames) and frames: the persistent
    launch reads the pressure weights of each step like the per-step launches."""
    scs, run = pkg.workloads.plate_pressure(nft=200)
    (ra, Ua, _), (rb, Ub, _) = run_both(pkg, scs, run, tile_elems=32, rows_per_block=2)
    for a, b in zip(ra, rb):
        np.testing.assert_array_equal(a["displ"], b["displ"])
        if run.frm_int > 0:
            np.testing.assert_array_equal(a["frames"], b["frames"])
    assert np.abs(Ua).max() > 0
    np.testing.assert_array_equal(Ua, Ub)
