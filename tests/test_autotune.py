"""Launch-shape autotuner and the batched-replica workload definition.

The chunk counts only split sums differently: tuned and heuristic shapes must
give the same forces (to rounding in FP64, to FP32 reordering in mixed mode).
"""
import collections

import numpy as np
import pytest


def test_replica_set_is_seeded_and_spans_the_configuration():
    from qtip4pf_water_gb300.workloads import replica_set

    a, b = replica_set(48), replica_set(48)
    assert a == b
    assert len(a) == 48
    assert set(x[0] for x in a) <= {64, 128, 216, 343, 512}
    assert set(x[1] for x in a) <= {8, 16, 32}
    assert len(collections.Counter(x[0] for x in a)) == 5
    assert all(250.0 <= x[2] < 350.0 for x in a)
    assert len(set(x[3] for x in a)) == 48  # every replica has its own start seed
    assert replica_set(49) != a


def test_block_standard_error_of_white_noise():
    from qtip4pf_water_gb300.workloads import block_se

    x = np.random.default_rng(3).standard_normal(100000)
    assert abs(block_se(x, 20) - 1.0 / np.sqrt(len(x))) < 0.4 / np.sqrt(len(x))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 1e-5)])
def test_autotuned_shapes_keep_the_forces(gpu_lib, precision, tol):
    import qtip4pf_water_gb300 as q

    st = q.seeded_start(216, 8, 298.0, seed=5)
    forces = []
    for tuned in (False, True):
        ctx = q.Context([q.system_desc(216, 8, st.box_bohr, propagator=q.TROTTER)], precision)
        ctx.systems[0].set_state(st.q, st.p)
        if tuned:
            t_heur, t_best = ctx.autotune(3)
            assert 0.0 < t_best <= t_heur
            n_rj, n_sc, n_kc = ctx.tuning()
            assert 0 <= n_rj <= 16 and 0 <= n_sc <= 32 and 0 <= n_kc <= 16
        ctx.init_forces()
        forces.append(ctx.systems[0].get_state()["fphys"])
        ctx.close()
    d = forces[1] - forces[0]
    assert np.sqrt(np.mean(d * d) / np.mean(forces[0] ** 2)) < tol


@pytest.mark.gpu
def test_fixed_tuning_is_checked_and_used(gpu_lib):
    import qtip4pf_water_gb300 as q

    st = q.seeded_start(64, 4, 298.0, seed=6)
    ctx = q.Context([q.system_desc(64, 4, st.box_bohr, propagator=q.TROTTER)], q.MIXED)
    ctx.systems[0].set_state(st.q, st.p)
    with pytest.raises(q.QtgError):
        ctx.set_tuning(17, 1, 1)
    ctx.set_tuning(1, 8, 3)
    assert ctx.tuning() == (1, 8, 3)
    ctx.init_forces()
    ctx.run_steps(3, is_nvt=True)
    ctx.sync()
    assert np.all(np.isfinite(ctx.systems[0].estimators()["conserved"]))
    ctx.close()
