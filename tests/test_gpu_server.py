"""The request executor (pm_server_*) on the GPU: results against the oracle,
cache reuse across requests, eviction under a small cap, Stokes requests."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from mymoonmd_gb300 import workloads as wl
from oracle import cd as ocd

pytestmark = pytest.mark.gpu


def db(precision="fp64", smoother="jacobi"):
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
    return d


def submit(srv, rq, tag, out):
    cf = m.cd_coeffs(rq["eps"], rq["b"], 0.0, True) if rq["kind"] == m.KIND_CD else None
    srv.submit(rq["kind"], rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], rq["elem"], cf,
               rq["nu"], out, tag)


def test_requests_match_oracle_and_reuse_cached_problems():
    reqs = [wl.cd_request(2, 32, 1, 0.1, (1.0, 0.0)), wl.cd_request(2, 32, 1, 0.5, (0.0, 0.7)),
            wl.cd_request(3, 8, 2, 0.2, (0.5, 0.5, 0.5)), wl.cd_request(2, 32, 1, 0.05, (0.6, 0.8))]
    outs = [np.empty(wl.dofs_of(r)) for r in reqs]
    srv = m.Server(0, 2, db(), None, int(8e9))
    try:
        for i, rq in enumerate(reqs):
            submit(srv, rq, i, outs[i])
        srv.drain()
        res = {r["tag"]: r for r in srv.poll(16)}
        assert sorted(res) == [0, 1, 2, 3]
        assert all(r["status"] == 0 for r in res.values()), res
        # a second round: every set-up is cached on the worker that serves it or not
        for i, rq in enumerate(reqs):
            submit(srv, rq, 10 + i, None)
        srv.drain()
        second = srv.poll(16)
        assert len(second) == 4 and all(r["status"] == 0 for r in second)
        assert sum(r["cache_hit"] for r in second) >= 2
        st = srv.stats()
        assert st["served"] == 8 and st["cached_bytes"] > 0
    finally:
        srv.close()
    for i, rq in enumerate(reqs):
        # the library's default rule: Gauss3 for Q1, Gauss4 for Q2
        o = ocd.OracleCD(rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], rq["elem"], rq["eps"],
                         rq["b"], 0.0, 3 if rq["elem"] == 1 else 4)
        o.assemble()
        o.build_mg(2, 2, 0.8, 1.0, "V")
        sol, it, resid, hist, st = o.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
        assert np.abs(outs[i] - sol).max() <= 1e-10 * np.abs(sol).max(), i
        assert abs(res[i]["iterations"] - it) <= 1


def test_small_cap_evicts_and_stokes_requests_run():
    reqs = [wl.cd_request(2, 64, 2, 0.1, (1.0, 0.0)), wl.cd_request(3, 16, 1, 0.1, (1.0, 0.0, 0.0)),
            wl.stokes_request(8), wl.cd_request(2, 64, 2, 0.2, (0.0, 1.0))]
    srv = m.Server(0, 1, db("mixed"), db("mixed", "nodal_vanka"), 40 * 2**20)
    try:
        for i, rq in enumerate(reqs):
            submit(srv, rq, i, None)
        srv.drain()
        res = srv.poll(16)
        assert len(res) == 4
        assert all(r["status"] == 0 for r in res), res
        st = srv.stats()
        assert st["evictions"] >= 1 and st["cached_bytes"] <= 40 * 2**20
    finally:
        srv.close()
