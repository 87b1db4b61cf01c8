"""Size-independent properties at the benchmark sizes, where the oracle cannot
run: the 512-plate batch (U{40..80}^2 order-5 elements, 232 M DOF, FP32 fused
structured kernel) and the 3D-solid plate of 120 x 120 x 8 hexahedra (18.4 M
DOF), over their first few hundred time steps.

* Linearity: every operation of a step is linear in the state and the
  excitation, and scaling by a power of two is exact in floating point for
  values in the normal range, so driving with 2 s(t) gives twice every signal
  up to what happens below it: the leading edge of each wave front starts
  below 2^-126, where the rounding does not scale, and grows by many orders
  of magnitude as the front arrives.  On the batch that leaves 5.7e-6 of the
  largest signal; the bound is 1e-4 (the FP32 error against FP64 is 1.8e-5 on
  the 20 x 20-element plate).
* Independence: a plate's signals in the full batch are bit-identical to a
  solo run of that plate with the same kernel configuration."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 300
LIN_TOL = 1e-4


@pytest.fixture(scope="module")
def full_batch(pkg):
    scs, run = pkg.workloads.batch(n=512, seed=0, nft=STEPS)
    plan = pkg.Plan(scs, run, precision=32, path=2, tile_elems=32, rows_per_block=32, steps_per_graph=50)
    assert plan.info["path"] == 2
    yield scs, run, plan
    plan.close()


def stacked(results):
    return np.concatenate([np.asarray(r["displ"]).ravel() for r in results])


def test_full_batch_is_linear(full_batch):
    scs, run, plan = full_batch
    sig = plan.signals()
    d1 = stacked(plan.forward(signals=sig))
    d2 = stacked(plan.forward(signals=2.0 * sig))
    scale = np.abs(d1).max()
    assert scale > 0 and np.isfinite(d2).all()
    ratio = np.abs(d2 - 2.0 * d1).max() / (2.0 * scale)
    assert ratio <= LIN_TOL, ratio


def test_full_batch_plates_equal_solo_runs(pkg, full_batch):
    scs, run, plan = full_batch
    batch = plan.forward()
    for s in (0, 255, 511):
        p1 = pkg.Plan([scs[s]], run, precision=32, path=2, tile_elems=32, rows_per_block=32)
        solo = p1.forward()[0]
        p1.close()
        assert np.abs(solo["displ"]).max() > 0
        np.testing.assert_array_equal(batch[s]["displ"], solo["displ"])


def test_fp32_error_on_benchmark_plates(pkg):
    """The metric's accuracy condition at the benchmark's plate sizes: four
    plates of 70-80^2 elements (the large end of the batch's U{40..80}) over
    the whole 0.4 ms (5 557 steps), the fused FP32 kernel in the benchmark's
    configuration against the engine's FP64 path (which equals the oracle to
    1e-10 where the oracle runs): the 8 sensor displacement signals and their
    velocities within 1e-3 relative L2 on every plate."""
    scs, run = pkg.workloads.batch(n=4, seed=3, nmin=70, nmax=80)
    assert run.nft - run.nn_first + 1 >= 5000
    p32 = pkg.Plan(scs, run, precision=32, path=2, tile_elems=32, rows_per_block=32, steps_per_graph=50)
    r32 = p32.forward()
    p32.close()
    p64 = pkg.Plan(scs, run, precision=64, path=0, steps_per_graph=50)
    r64 = p64.forward()
    p64.close()
    for s in range(len(scs)):
        a, b = r32[s]["displ"], r64[s]["displ"]
        assert np.abs(b).max() > 0
        e_d = np.linalg.norm(a - b) / np.linalg.norm(b)
        va, vb = a[2:] - a[:-2], b[2:] - b[:-2]
        e_v = np.linalg.norm(va - vb) / np.linalg.norm(vb)
        assert e_d <= 1e-3 and e_v <= 1e-3, (s, e_d, e_v)


def test_full_solid_plate_is_linear(pkg):
    scs, run = pkg.workloads.solid_plate(nft=STEPS)
    plan = pkg.SolidPlan(scs, run, precision=32, steps_per_graph=50)
    try:
        sig = plan.signals()
        d1 = stacked(plan.forward(signals=sig))
        d2 = stacked(plan.forward(signals=2.0 * sig))
    finally:
        plan.close()
    scale = np.abs(d1).max()
    assert scale > 0 and np.isfinite(d2).all()
    ratio = np.abs(d2 - 2.0 * d1).max() / (2.0 * scale)
    assert ratio <= LIN_TOL, ratio
