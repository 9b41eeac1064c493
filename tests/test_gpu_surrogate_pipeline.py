"""The learned centroid correction end to end at a small size: constrained-PIMD
data on the device stepper, training on the tensor cores, the gain over the
classical force on held-out configurations, and the correction inside a P = 1
force evaluation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(gpu_lib):
    pytest.importorskip("torch")
    from qtip4pf_water_gb300 import surrogate as sg

    ds = sg.generate(n_mols=64, n_beads=8, n_configs=64, replicas=16, equil_steps=400, sample_every=100,
                     constrained_steps=600, seed=3)
    train, test = ds.split(48)
    X, T = sg.features(train)
    model = sg.Correction(seed=1)
    model.fit(X, T, steps=600, lr=3e-3, lr_final=3e-4)
    return sg, ds, train, test, model


def test_correction_beats_the_classical_force_on_held_out_configs(trained):
    sg, ds, train, test, model = trained
    assert np.all(np.isfinite(ds.fmean)) and np.all(np.isfinite(ds.fclass))
    # the quantum mean centroid force differs from the classical force
    assert np.sqrt(np.mean((ds.fmean - ds.fclass) ** 2)) > 1e-3 * np.sqrt(np.mean(ds.fmean ** 2))
    ev_train, ev_test = model.evaluate(train), model.evaluate(test)
    assert model.history[-1][1] < 0.8 * model.history[0][1]
    assert ev_train["rms_rel_err_corrected"] < ev_train["rms_rel_err_classical"]
    assert ev_test["rms_rel_err_corrected"] < ev_test["rms_rel_err_classical"], ev_test


def test_attached_correction_matches_the_host_prediction(trained, gpu_lib):
    sg, ds, train, test, model = trained
    q = gpu_lib
    c = test.centroids[0]
    ctx = q.Context([q.system_desc(64, 1, ds.box, propagator=q.TROTTER, thermostat=q.PILE_L)], q.MIXED)
    s = ctx.systems[0]
    s.set_state(c)
    model.attach(s)
    ctx.init_forces()
    got = s.get_state()["fphys"]
    sub = sg.Dataset(64, ds.box, test.centroids[:1], test.fmean[:1], test.fclass[:1], test.meta)
    want = test.fclass[0] + model.lab_corrections(sub)[0]
    corr = want - test.fclass[0]
    assert np.abs(got - want).max() < 2e-3 * np.abs(corr).max() + 1e-6
    # steps run with the correction in the graph; detaching restores the classical force
    ctx.run_steps(5, is_nvt=True)
    ctx.sync()
    assert np.all(np.isfinite(s.get_state()["q"]))
    s.set_state(c)
    s.detach_surrogate()
    ctx.init_forces()
    assert np.abs(s.get_state()["fphys"] - test.fclass[0]).max() < 1e-6 * np.abs(test.fclass[0]).max()
