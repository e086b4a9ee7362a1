"""The serving form: convection-diffusion requests of one set-up batched into
single launches (batch lanes), Stokes requests on the worker pool, one HBM
cap for all of them.

  * continuous batching: a request's result is the same, bit for bit, alone
    and in a mix of concurrent requests (other coefficients of its set-up,
    other set-ups, Stokes requests), in the FP64 and in the mixed form; the
    same holds for Stokes requests;
  * the lane's batched FP64 results match the oracle within 1e-10;
  * a Stokes problem cached for its set-up takes each request's viscosity;
  * admission by footprint: under a cap that holds about two problems every
    request completes and the server's memory ends under the cap.
"""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from mymoonmd_gb300 import workloads as wl
from oracle import cd as ocd

pytestmark = pytest.mark.gpu


def db(precision="fp64", smoother="jacobi", slots=8):
    d = m.ParameterDatabase.solve_path_database()
    d["solver_type"] = "iterative"
    d["iterative_solver_type"] = "fgmres"
    d["preconditioner"] = "multigrid"
    d["residual_tolerance"] = 0.0
    d["residual_reduction"] = 1e-10
    d["max_n_iterations"] = 200
    d["gmres_restart"] = 20
    d["multigrid_smoother"] = smoother
    d["multigrid_smoother_coarse"] = "direct_solve"
    d["jacobi_damp"] = 0.8
    d["multigrid_vanka_damp_factor"] = 1.0
    d["multigrid_n_pre_smooth"] = 2 if smoother == "jacobi" else 1
    d["multigrid_n_post_smooth"] = 2 if smoother == "jacobi" else 1
    d["gpu_precision"] = precision
    d["gpu_mixed_fallback"] = 0
    d.add("gpu_batch_slots", slots)
    return d


def stokes_db(precision="fp64"):
    d = db(precision, "nodal_vanka")
    d["multigrid_smoother_coarse"] = "nodal_vanka_jacobi"
    d["multigrid_vanka_damp_factor"] = 0.8
    return d


def submit(srv, rq, tag, out):
    cf = m.cd_coeffs(rq["eps"], rq["b"], 0.0, True) if rq["kind"] == m.KIND_CD else None
    srv.submit(rq["kind"], rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], rq["elem"], cf,
               rq["nu"], out, tag)


def run(srv, reqs):
    outs = [np.zeros(wl.dofs_of(r)) for r in reqs]
    for i, rq in enumerate(reqs):
        submit(srv, rq, i, outs[i])
    srv.drain()
    res = {r["tag"]: r for r in srv.poll(4096)}
    return outs, res


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_result_is_the_same_alone_and_in_the_mix(precision):
    probe_cd = wl.cd_request(3, 8, 2, 0.1, (1.0, 0.5, 0.25))
    probe_st = wl.stokes_request(8)
    mix = [wl.cd_request(3, 8, 2, 10 ** (-k / 6), (np.cos(k), np.sin(k), 0.3)) for k in range(9)]
    mix += [wl.cd_request(2, 32, 1, 0.05 * (k + 1), (1.0, 0.2 * k)) for k in range(5)]
    mix += [wl.stokes_request(8), wl.stokes_request(8, 2.0)]
    srv = m.Server(0, 2, db(precision), stokes_db(precision), int(40e9))
    try:
        alone_cd, res_a = run(srv, [probe_cd])
        alone_st, res_s = run(srv, [probe_st])
        assert res_a[0]["status"] == 0 and res_s[0]["status"] == 0
        reqs = mix[:4] + [probe_cd] + mix[4:11] + [probe_st] + mix[11:]
        outs, res = run(srv, reqs)
        assert all(r["status"] == 0 for r in res.values()), {k: r["status"] for k, r in res.items()}
        i_cd, i_st = reqs.index(probe_cd), reqs.index(probe_st)
        assert np.array_equal(outs[i_cd], alone_cd[0])
        assert res[i_cd]["iterations"] == res_a[0]["iterations"]
        assert np.array_equal(outs[i_st], alone_st[0])
        # the batch lane served requests together: more than one of the 3D
        # requests shares a lane (worker index above the pool's)
        lanes = {r["worker"] for k, r in res.items() if reqs[k]["kind"] == m.KIND_CD}
        assert min(lanes) >= 2
    finally:
        srv.close()


def test_batched_lane_results_match_the_oracle():
    reqs = [wl.cd_request(2, 32, 1, 0.1, (1.0, 0.0)), wl.cd_request(2, 32, 1, 0.5, (0.0, 0.7)),
            wl.cd_request(2, 32, 1, 0.05, (0.6, 0.8)), wl.cd_request(3, 8, 2, 0.2, (0.5, 0.5, 0.5))]
    srv = m.Server(0, 1, db(), None, int(8e9))
    try:
        outs, res = run(srv, reqs)
    finally:
        srv.close()
    for i, rq in enumerate(reqs):
        assert res[i]["status"] == 0
        # the library's default rule: Gauss3 for Q1, Gauss4 for Q2
        o = ocd.OracleCD(rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], rq["elem"], rq["eps"],
                         rq["b"], 0.0, 3 if rq["elem"] == 1 else 4)
        o.assemble()
        o.build_mg(2, 2, 0.8, 1.0, "V")
        sol, it, resid, hist, st = o.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
        assert np.abs(outs[i] - sol).max() <= 1e-10 * np.abs(sol).max(), i
        assert abs(res[i]["iterations"] - it) <= 1


def test_cached_stokes_problem_takes_each_requests_viscosity():
    srv = m.Server(0, 1, db(), stokes_db(), int(8e9))
    try:
        outs, res = run(srv, [wl.stokes_request(8, 1.0), wl.stokes_request(8, 3.0)])
        assert res[0]["status"] == 0 and res[1]["status"] == 0 and res[1]["cache_hit"] == 1
    finally:
        srv.close()
    ctx = m.Context(0)
    try:
        for k, nu in enumerate((1.0, 3.0)):
            disc = m.Discretization(m.GEO_CUBE_TETRA, 2, 2, 3, m.KIND_STOKES, 12)
            d = stokes_db()
            d["multigrid_n_levels"] = 3
            p = m.StokesProblem(ctx, disc, nu, d)
            p.assemble()
            p.solve()
            assert np.array_equal(p.solution(), outs[k])
            p.close()
            disc.close()
    finally:
        ctx.close()


def test_admission_under_a_small_cap():
    reqs = [wl.cd_request(3, 16, 2, 0.1 * (k + 1), (1.0, 0.0, 0.0)) for k in range(6)]
    reqs += [wl.cd_request(2, 64, 2, 0.1 * (k + 1), (0.0, 1.0)) for k in range(6)]
    # the footprint of one lane with one problem, per set-up
    fp = []
    for rq in (reqs[0], reqs[6]):
        srv = m.Server(0, 1, db("mixed", slots=4), None, int(40e9))
        try:
            run(srv, [rq])
            fp.append(srv.stats()["cached_bytes"])
        finally:
            srv.close()
    # room for the larger lane and a part of the other: requests must wait
    # for slots and for memory
    cap = max(fp) + min(fp) // 2
    srv = m.Server(0, 1, db("mixed", slots=4), None, cap)
    try:
        outs, res = run(srv, reqs)
        assert len(res) == len(reqs)
        assert all(r["status"] == 0 for r in res.values()), res
        st = srv.stats()
        assert st["cached_bytes"] <= cap
    finally:
        srv.close()
