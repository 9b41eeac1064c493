"""Same inputs, same seed, same bits: the device stepper's trajectory does not
depend on the order in which blocks run. The system sums that steer the dynamics
(the centroid kinetic energy behind the PILE-G rescale) and the thermostat heat
are reduced in a fixed order; the force planes are written, never accumulated
atomically."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_stepper_trajectory_is_reproducible(gpu_lib, precision):
    q = gpu_lib
    prec = q.MIXED if precision == "mixed" else q.FP64
    st = q.seeded_start(64, 8, 298.0, seed=17)
    runs = []
    for _ in range(2):
        ctx = q.Context([q.system_desc(64, 8, st.box_bohr, propagator=q.TROTTER, thermostat=q.PILE_G, seed=17)],
                        prec)
        ctx.systems[0].set_state(st.q, st.p)
        ctx.init_forces()
        ctx.run_steps(25, is_nvt=True)
        ctx.sync()
        g = ctx.systems[0].get_state()
        est = ctx.systems[0].estimators()
        runs.append((g["q"], g["p"], g["fphys"], est["heat"] if "heat" in est else None))
        ctx.close()
    for a, b in zip(runs[0][:3], runs[1][:3]):
        assert np.array_equal(a, b)
    if runs[0][3] is not None:
        assert np.array_equal(runs[0][3], runs[1][3])
