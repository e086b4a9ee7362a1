"""Synthetic request streams: the batched stream of independent
convection-diffusion solves and the serving mix of convection-diffusion and
Stokes requests. Every request is a dict with the fields of pm_request
(kind, geometry, root_n, n_refine, n_levels, elem, eps, b, nu) plus its mesh
size; the draws are seeded and reproducible.
"""
from __future__ import annotations

import math

import numpy as np

from .core import GEO_CUBE_HEXA, GEO_CUBE_TETRA, GEO_SQUARE_QUAD, KIND_CD, KIND_STOKES


def mesh_for(dim: int, cells: int) -> tuple[int, int, int]:
    """(geometry, root_n, n_refine) of a uniform mesh with `cells` cells per side:
    a power of two refines one root cell, 24 refines a 3 x 3 (x 3) root mesh"""
    geo = GEO_SQUARE_QUAD if dim == 2 else GEO_CUBE_HEXA
    root = 3 if cells % 3 == 0 else 1
    r = int(round(math.log2(cells // root)))
    if root * (1 << r) != cells:
        raise ValueError(f"{cells} cells per side is neither 2^k nor 3 * 2^k")
    return geo, root, r


def cd_levels(dim: int, cells: int) -> int:
    """multigrid levels down to 4 (2D) or 2-3 (3D) cells per side"""
    floor = 4 if dim == 2 else 2
    geo, root, r = mesh_for(dim, cells)
    levels = 1
    c = cells
    while c % 2 == 0 and c // 2 >= floor and levels <= r:
        c //= 2
        levels += 1
    return levels


def cd_request(dim: int, cells: int, elem: int, eps: float, b) -> dict:
    geo, root, r = mesh_for(dim, cells)
    return dict(kind=KIND_CD, geometry=geo, root_n=root, n_refine=r, n_levels=cd_levels(dim, cells), elem=elem,
                eps=float(eps), b=tuple(float(x) for x in b) + (0.0,) * (3 - len(b)), nu=1.0, dim=dim,
                cells=cells)


def stokes_request(cubes: int, nu: float = 1.0) -> dict:
    """P2/P1 on `cubes`^3 cubes x 6 tetrahedra, three levels (cubes/4, cubes/2, cubes)"""
    if cubes % 4:
        raise ValueError("Stokes meshes need cubes per side divisible by 4 (three levels)")
    root = cubes // 4
    return dict(kind=KIND_STOKES, geometry=GEO_CUBE_TETRA, root_n=root, n_refine=2, n_levels=3, elem=12, eps=1.0,
                b=(0.0, 0.0, 0.0), nu=nu, dim=3, cells=cubes)


def stream_requests(n: int = 512, seed: int = 0) -> list[dict]:
    """the batched stream: per request, in this order of draws from
    numpy.random.default_rng(seed): dimension 2 or 3 (p = 1/2); cells per
    side from {32, 64, 128, 256} (2D) or {8, 16, 24, 32} (3D); Q1 or Q2
    (p = 1/2); eps log-uniform in [1e-3, 1]; b a uniformly random unit vector
    times a magnitude uniform in [0, 1]"""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        dim = int(rng.choice([2, 3]))
        cells = int(rng.choice([32, 64, 128, 256] if dim == 2 else [8, 16, 24, 32]))
        elem = int(rng.choice([1, 2]))
        eps = float(10.0 ** rng.uniform(-3.0, 0.0))
        d = rng.standard_normal(dim)
        d /= np.linalg.norm(d)
        b = d * rng.uniform(0.0, 1.0)
        out.append(cd_request(dim, cells, elem, eps, b))
    return out


def serving_requests(rate: float, duration_s: float, seed: int = 0, cd_share: float = 0.7) -> list[dict]:
    """Poisson arrivals at `rate` per second over `duration_s`: 70% 3D Q2
    convection-diffusion (cells per side from {8, 16, 24, 32}, eps and b drawn
    as in the batched stream), 30% Stokes P2/P1 (cubes per side from
    {8, 12, 16, 24}); each request carries its arrival time `t` in seconds"""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration_s:
            break
        if rng.uniform() < cd_share:
            cells = int(rng.choice([8, 16, 24, 32]))
            eps = float(10.0 ** rng.uniform(-3.0, 0.0))
            d = rng.standard_normal(3)
            d /= np.linalg.norm(d)
            rq = cd_request(3, cells, 2, eps, d * rng.uniform(0.0, 1.0))
        else:
            rq = stokes_request(int(rng.choice([8, 12, 16, 24])))
        rq["t"] = t
        out.append(rq)
    return out


def dofs_of(rq: dict) -> int:
    """number of DOFs of a request (all of them, Dirichlet included)"""
    c = rq["cells"]
    if rq["kind"] == KIND_STOKES:
        return 3 * (2 * c + 1) ** 3 + (c + 1) ** 3
    k = rq["elem"]
    return (k * c + 1) ** rq["dim"]
