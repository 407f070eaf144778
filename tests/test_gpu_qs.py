"""GPU quasi-static Newton (RNPBond) against the oracle's restatement.

Both stop at ||r|| <= 1e-8 ||r(previous-step guess)||; converged states agree
to well below the displacement scale, and the broken-bond sets match."""
import numpy as np
import pytest

from nlmech_gb300 import configs

pytestmark = pytest.mark.gpu


def pairs(rowptr, cols, broken):
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    sel = broken.astype(bool)
    return set(zip(rows[sel].tolist(), cols[sel].tolist()))


def test_qs_elastic_steps_match_oracle(gpu, oracle):
    """Below the fracture load: identical algorithm, states equal to ~1e-9."""
    p = configs.qs_plate(48, h=5e-4, du=4e-8)
    q = gpu.QSModel(p, gpu.qs_params(lin_tol=1e-6))
    o = oracle.OracleQSR(p, lin_tol=1e-6)
    for k in range(6):
        s = q.load_step()
        so = o.load_step()
        assert s["res_final"] <= 1e-8 * s["res_plain"]
        assert so["res_final"] <= 1e-8 * so["res_plain"]
        assert s["res_plain"] == pytest.approx(so["res_plain"], rel=1e-9)
        assert s["newton_iters"] == so["newton_iters"]
        u, uo = q.state(), o.state()
        assert np.abs(u - uo).max() <= 1e-9 * np.abs(uo).max()


def test_qs_fracture_steps_match_oracle(gpu, oracle):
    """Crack growth during Newton: converged states and broken-bond sets agree.
    Bonds break at intermediate Newton iterates, so the converged state depends
    on the iterates; the GPU's Krylov solve runs in FP32 and the oracle's in
    FP64, which moves a few break decisions (at most 1 % of the broken bonds)
    and the displacement by up to 1 % relative L2."""
    p = configs.qs_plate(48, h=5e-4, du=1e-6)
    prm = dict(max_newton=60)
    q = gpu.QSModel(p, gpu.qs_params(lin_tol=1e-6, **prm))
    o = oracle.OracleQSR(p, lin_tol=1e-6, **prm)
    rowptr, cols = oracle.neighbors(p.x, p.horizon)
    for k in range(4):
        s = q.load_step()
        so = o.load_step()
        assert s["res_final"] <= 1e-8 * s["res_plain"], (k, s)
        assert so["res_final"] <= 1e-8 * so["res_plain"], (k, so)
    bo = pairs(rowptr, cols, o.bond_state())
    assert len(bo) > 1000
    assert len(pairs(rowptr, cols, q.bond_state()) ^ bo) <= 0.01 * len(bo)
    u, uo = q.state(), o.state()
    assert np.linalg.norm(u - uo) <= 1e-2 * np.linalg.norm(uo)


def test_qs_guess_and_fallback(gpu):
    p = configs.qs_plate(40, h=5e-4, du=2e-6)
    q = gpu.QSModel(p)
    q.load_step()
    u1 = q.state()
    # a guess far worse than the previous step is rejected
    s = q.load_step(guess=u1 + 1e-3)
    assert s["used_guess"] == 0 and s["res_start"] == s["res_plain"]
    # so is one no better than the plain start (the previous state itself)
    q4 = gpu.QSModel(p)
    q4.load_step()
    s4 = q4.load_step(guess=q4.state())
    assert s4["used_guess"] == 0
    # the converged answer of the same (elastic) step is accepted and needs
    # no iteration
    p = configs.qs_plate(40, h=5e-4, du=2e-8)
    q2 = gpu.QSModel(p)
    q2.load_step()
    q2.load_step()
    u2 = q2.state()
    q3 = gpu.QSModel(p)
    q3.load_step()
    s3 = q3.load_step(guess=u2)
    assert s3["used_guess"] == 1
    assert s3["newton_iters"] <= 1


def test_qs_single_launch_krylov_matches_two_launch(gpu):
    """The FP32 Krylov solve in one cooperative launch (grid barriers between
    its phases, convergence tested every iteration) and the same solve in two
    launches per iteration reach the same Newton solutions: every load step
    converges to the 1e-8 relative residual in both, with equal broken bonds
    and displacements equal to the Newton tolerance."""
    p = configs.qs_plate(48, h=5e-4, du=1e-6)
    qa = gpu.QSModel(p, gpu.qs_params(lin_tol=1e-6, max_newton=60, krylov_launch=1))
    qb = gpu.QSModel(p, gpu.qs_params(lin_tol=1e-6, max_newton=60, krylov_launch=0))
    for k in range(4):
        sa, sb = qa.load_step(), qb.load_step()
        assert sa["res_final"] <= 1e-8 * sa["res_plain"], (k, sa)
        assert sb["res_final"] <= 1e-8 * sb["res_plain"], (k, sb)
    ua, ub = qa.state(), qb.state()
    assert np.linalg.norm(ua - ub) <= 1e-2 * np.linalg.norm(ub)
    ba, bb = qa.bond_state(), qb.bond_state()
    assert np.count_nonzero(ba != bb) <= 0.01 * max(np.count_nonzero(bb), 1)


def test_qs_barrier_wait_runs_out_with_status(gpu):
    """Each grid-barrier wait of the single-launch solve is bounded: with
    every barrier made to wait for one block that does not exist, each wait
    runs out after 50 ms, the launch ends and the load step fails with
    NLM_ERR_TIMEOUT; the device stays usable for the next model."""
    p = configs.qs_plate(40, h=5e-4, du=1e-6)
    bad = gpu.QSModel(p, gpu.qs_params(krylov_launch=1, wait_limit_s=0.05, barrier_extra=1))
    with pytest.raises(gpu.NLMError) as e:
        bad.load_step()
    assert e.value.code == 4  # NLM_ERR_TIMEOUT
    bad.close()
    good = gpu.QSModel(p, gpu.qs_params())
    s = good.load_step()
    assert s["res_final"] <= 1e-8 * s["res_plain"]
