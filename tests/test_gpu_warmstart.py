"""Learned warm start end to end on a small plate: data from the plain
solver, BF16 training on the GPU, then learned vs plain load steps on a
geometry outside the training seeds, both converged to the same tolerance."""
import numpy as np
import pytest

from nlmech_gb300 import configs

pytestmark = pytest.mark.gpu


def test_warm_start_small_plate(gpu):
    from nlmech_gb300 import warmstart as ws
    params = gpu.qs_params(max_newton=300)
    runs = [ws.run_steps(configs.qs_training_geometry(s, nx=48), 15, params, record=True)
            for s in (0, 1, 2)]
    X = np.concatenate([r["X"] for r in runs])
    T = np.concatenate([r["T"] for r in runs])
    assert 0.9 * 3 * 15 * 48 * 48 <= X.shape[0] <= 3 * 15 * 48 * 48
    assert X.shape[1] == ws.N_FEAT and T.shape == (X.shape[0], ws.N_OUT)
    assert np.abs(X[:, 2:6]).max() <= ws.FEATURE_CLIP and np.abs(T).max() <= ws.TARGET_CLIP
    assert np.all(np.isfinite(X)) and np.all(np.isfinite(T))
    m = gpu.MLP(ws.N_FEAT, ws.HIDDEN, ws.LAYERS, ws.N_OUT, seed=3)
    m.set_data(X, T)
    losses = m.train(8, batch=1024, lr=1e-3, seed=0)
    assert losses[-1] < losses[0]
    p = configs.qs_training_geometry(7, nx=48)
    ra = ws.run_steps(p, 15, params)
    rb = ws.run_steps(p, 15, params, model=m)
    a, b = ws.summary(ra), ws.summary(rb)
    assert a["all_steps_converged"] and b["all_steps_converged"]
    assert b["guess_used"] >= 5
    # an accepted guess never starts from a larger linearised residual than
    # the plain start, and every step still reaches the same tolerance
    for st in rb["stats"]:
        if st["used_guess"]:
            assert st["res_start"] <= st["res_plain"]
        assert st["res_final"] <= 1e-8 * st["res_plain"]


def test_trained_network_cuts_newton_work(gpu):
    """The committed network (trained on the plain solver's load steps of 20
    seeded pre-crack geometries) on the 200 x 200 plate with the centred
    0.2 W pre-crack, a geometry outside its training seeds, 100 load steps:
    every step of both runs converges to the same 1e-8 relative residual,
    the learned start needs at least 1.5x fewer Newton iterations and Krylov
    iterations and at most half the wall time of the plain previous-step
    start, and it ends in the plain run's state (QuasiStaticModel.cpp:526-594).
    Both runs use the same Newton-Krylov settings (the evaluation's forcing
    term)."""
    from nlmech_gb300 import warmstart as ws
    model = ws.load_model()
    p = configs.config4()
    params = gpu.qs_params(max_newton=500, lin_tol_gamma=ws.LIN_TOL_GAMMA)
    ra = ws.run_steps(p, 100, params)
    rb = ws.run_steps(p, 100, params, model=model)
    a, b = ws.summary(ra), ws.summary(rb)
    print("plain", a, "learned", b)
    assert a["all_steps_converged"] and b["all_steps_converged"]
    assert a["newton_iters"] >= 1.5 * b["newton_iters"]
    assert a["cg_iters"] >= 1.5 * b["cg_iters"]
    assert 2.0 * rb["wall_s"] <= ra["wall_s"], (ra["wall_s"], rb["wall_s"])
    du = np.linalg.norm(rb["u"] - ra["u"]) / np.linalg.norm(ra["u"])
    assert du <= 1e-6, du
    for st in rb["stats"]:
        assert st["res_final"] <= 1e-8 * st["res_plain"]
