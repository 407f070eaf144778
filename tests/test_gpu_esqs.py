"""QuasiStaticModel<ElasticState> on the GPU (nlm_esqs_*) against the
reference's stored results (examples/qsModel/{1D,2D}/output_res.vtu, decoded
into tests/golden/qs_*.npz) at the reference test's own bar (L2 < 1e-7 on
Displacement, tools/dc/src/fdSimple.cpp:164-176), and against the oracle's
restatement over several load steps with force and displacement loading
(1e-8 relative: both solve each Newton step to a tight linear tolerance, the
oracle by LU, the GPU by BiCGSTAB)."""
import numpy as np
import pytest

from nlmech_gb300 import abi, configs
from nlmech_gb300.decks import BC, MaterialDeck, Problem
from test_oracle import _golden_problem, _l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["qs_1d", "qs_2d"])
@pytest.mark.parametrize("jac", [0, 1])
def test_esqs_matches_reference_results(gpu, name, jac):
    p, z, deck = _golden_problem(name)
    prm = gpu.esqs_params(max_iters=deck["max_iters"], tol=deck["tol"], jacobian=jac,
                          perturbation=deck["perturbation"],
                          dt=deck["final_time"] / deck["time_steps"])
    q = gpu.ESQSModel(p, prm)
    iters, lin, res = q.solve(deck["time_steps"])
    assert res < deck["tol"], (iters, res)
    u, f = q.get()
    assert _l2(u, z["displacement"]) < deck["compare_tol"], _l2(u, z["displacement"])
    assert _l2(f, z["force"]) < 1e-6 * max(1.0, np.abs(z["force"]).max())


def _loaded_plate():
    x, vol = configs.grid2d(14, 10, 0.1, jitter=0.05, seed=2)
    mat = MaterialDeck(kind="ElasticState", density=1200.0, K=4000.0, G=1500.0)
    ubc = [BC(region="rectangle", x1=-0.01, x2=0.12, y1=-0.01, y2=1.01, direction=[1, 2],
              time_fn="constant", time_params=[0.0], spatial_fn="constant",
              spatial_params=[1.0]),
           BC(region="rectangle", x1=1.28, x2=1.41, y1=-0.01, y2=1.01, direction=[2],
              time_fn="linear", time_params=[0.01], spatial_fn="constant",
              spatial_params=[1.0])]
    fbc = [BC(region="rectangle", x1=1.28, x2=1.41, y1=-0.01, y2=1.01, direction=[1],
              time_fn="linear", time_params=[1.0], spatial_fn="constant",
              spatial_params=[-50.0])]
    return Problem(dim=2, x=x, volume=vol, horizon=0.3, mesh_size=0.1, material=mat,
                   ubc=ubc, fbc=fbc)


def test_esqs_load_steps_match_oracle(gpu, oracle):
    p = _loaded_plate()
    dt = 0.25
    prm_o = oracle.QSParams(jacobian=1, solver=0, max_iters=50, tol=1e-9, tol_relative=0,
                            perturbation=1e-7, lin_max_iters=1000, lin_tol=1e-12, dt=dt)
    o = oracle.OracleQS(p, prm_o)
    q = gpu.ESQSModel(p, gpu.esqs_params(max_iters=50, tol=1e-9, jacobian=1, dt=dt))
    for step in range(3):
        io, ro = o.solve(1)
        ig, lg, rg = q.solve(1)
        assert rg < 1e-9 and ro < 1e-9, (step, rg, ro)
        uo, fo = o.get()
        ug, fg = q.get()
        assert np.abs(ug - uo).max() <= 1e-8 * np.abs(uo).max(), step
        assert np.abs(fg - fo).max() <= 1e-6 * max(1e-12, np.abs(fo).max()), step
    assert np.abs(uo).max() > 0


def test_esqs_rejects_other_inputs(gpu):
    p = configs.rnp_plate(10, 1e-3, 3, 0.0, 0.1, 1e-8, 10)
    with pytest.raises(gpu.NLMError):
        gpu.ESQSModel(p)
    q = _loaded_plate()
    with pytest.raises(gpu.NLMError):
        gpu.ESQSModel(q, gpu.esqs_params(tol=-1.0))
