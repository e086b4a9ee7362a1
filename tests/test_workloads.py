"""Request generators of the batched stream and the serving mix (host only)."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from mymoonmd_gb300 import workloads as wl


def test_stream_is_reproducible_and_in_range():
    a, b = wl.stream_requests(512, 0), wl.stream_requests(512, 0)
    assert a == b
    assert wl.stream_requests(8, 1) != wl.stream_requests(8, 0)
    dims = [r["dim"] for r in a]
    assert 200 < dims.count(2) < 312
    for r in a:
        allowed = [32, 64, 128, 256] if r["dim"] == 2 else [8, 16, 24, 32]
        assert r["cells"] in allowed and r["elem"] in (1, 2)
        assert 1e-3 <= r["eps"] <= 1.0
        assert np.linalg.norm(r["b"]) <= 1.0 + 1e-12
        assert r["geometry"] == (m.GEO_SQUARE_QUAD if r["dim"] == 2 else m.GEO_CUBE_HEXA)


@pytest.mark.parametrize("dim,cells,geo,root,nref,levels", [
    (2, 32, m.GEO_SQUARE_QUAD, 1, 5, 4), (2, 256, m.GEO_SQUARE_QUAD, 1, 8, 7),
    (3, 8, m.GEO_CUBE_HEXA, 1, 3, 3), (3, 24, m.GEO_CUBE_HEXA, 3, 3, 4), (3, 32, m.GEO_CUBE_HEXA, 1, 5, 5)])
def test_mesh_and_levels(dim, cells, geo, root, nref, levels):
    assert wl.mesh_for(dim, cells) == (geo, root, nref)
    assert wl.cd_levels(dim, cells) == levels


@pytest.mark.parametrize("rq", [wl.cd_request(2, 32, 2, 0.1, (1.0, 0.0)), wl.cd_request(3, 24, 1, 0.1, (1, 0, 0)),
                                wl.stokes_request(8), wl.stokes_request(12)])
def test_dof_counts_match_the_setup(rq):
    d = m.Discretization(rq["geometry"], rq["root_n"], rq["n_refine"], rq["n_levels"], rq["kind"], rq["elem"])
    fin = rq["n_levels"] - 1
    n = d.level_info(fin)["n_dofs"]
    if rq["kind"] == m.KIND_STOKES:
        n = 3 * n + d.level_info(fin, 1)["n_dofs"]
    assert n == wl.dofs_of(rq)


def test_serving_arrivals():
    reqs = wl.serving_requests(200.0, 5.0, seed=1)
    assert 800 < len(reqs) < 1200
    ts = [r["t"] for r in reqs]
    assert ts == sorted(ts) and ts[-1] < 5.0
    share = sum(r["kind"] == m.KIND_CD for r in reqs) / len(reqs)
    assert 0.62 < share < 0.78
