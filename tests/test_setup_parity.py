"""Host set-up of the library (mesh hierarchy, DOF numbering, CSR structure,
prolongation) against the oracle's independent restatement. These calls are
host-only inside libpmgpu.so and need no GPU. Integer data must agree
bit-for-bit."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd
from oracle import refsetup

CASES = [
    (m.GEO_SQUARE_QUAD, 1, 4, 3, 1),
    (m.GEO_SQUARE_QUAD, 1, 3, 2, 2),
    (m.GEO_SQUARE_QUAD, 3, 2, 2, 1),
    (m.GEO_CUBE_HEXA, 1, 3, 3, 1),
    (m.GEO_CUBE_HEXA, 1, 3, 2, 2),
    (m.GEO_CUBE_HEXA, 3, 1, 2, 2),
]


@pytest.mark.parametrize("geo,root,nref,nlev,elem", CASES)
def test_numbering_and_structure_bit_exact(geo, root, nref, nlev, elem):
    d = m.Discretization(geo, root, nref, nlev, m.KIND_CD, elem)
    ref = refsetup.cd_levels(geo, root, nref, nlev, elem)
    for l in range(nlev):
        info = d.level_info(l)
        assert info["n_dofs"] == ref[l].n_dofs and info["n_active"] == ref[l].n_active
        assert np.array_equal(d.dofmap(l), ref[l].dofmap)
        rp, ci = d.structure(l)
        assert np.array_equal(rp, ref[l].row_ptr)
        assert np.array_equal(ci, ref[l].cols)
        assert np.array_equal(d.cell_vertices(l), ref[l].verts)


@pytest.mark.parametrize("geo,root,nref,nlev,elem", CASES)
def test_prolongation_matches_oracle_transfer(geo, root, nref, nlev, elem):
    d = m.Discretization(geo, root, nref, nlev, m.KIND_CD, elem)
    ref = refsetup.cd_levels(geo, root, nref, nlev, elem)
    dim = 2 if geo == m.GEO_SQUARE_QUAD else 3
    rng = np.random.default_rng(1)
    for l in range(nlev - 1):
        rp, ci, v, nr, nc = d.prolongation(l)
        c, f = ref[l], ref[l + 1]
        xc = rng.standard_normal(c.n_dofs)
        P = np.zeros((nr, nc))
        for i in range(nr):
            P[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        # prolongation: the active fine rows (GridTransfer::Prolongate + damped add)
        ora = ocd.transfer(dim, elem, c, f, xc, True)
        assert np.allclose((P @ xc)[: f.n_active], ora[: f.n_active], rtol=0, atol=1e-13)
        # restriction of a defect with zero non-active entries (always the case in the cycle)
        xf = rng.standard_normal(f.n_dofs)
        xf[f.n_active:] = 0.0
        orr = ocd.transfer(dim, elem, c, f, xf, False)
        assert np.allclose(P.T @ xf, orr, rtol=0, atol=1e-12)


def test_config_sizes():
    """DOF and nonzero counts of the 2D Q1 128^2 and 3D Q2 32^3 workloads"""
    d = m.Discretization(m.GEO_SQUARE_QUAD, 1, 7, 4, m.KIND_CD, 1)
    assert [d.level_info(l)["n_dofs"] for l in range(4)] == [289, 1089, 4225, 16641]
    assert d.level_info(3)["nnz"] == 145673 and d.level_info(3)["n_active"] == 16129
    d = m.Discretization(m.GEO_CUBE_HEXA, 1, 5, 4, m.KIND_CD, 2)
    assert [d.level_info(l)["n_dofs"] for l in range(4)] == [729, 4913, 35937, 274625]
    assert [d.level_info(l)["nnz"] for l in range(4)] == [20069, 206917, 1867013, 15837829]


def test_invalid_setup_reports_error():
    with pytest.raises(m.PmError):
        m.Discretization(m.GEO_CUBE_TETRA, 1, 2, 2, m.KIND_CD, 2)
    with pytest.raises(m.PmError):
        m.Discretization(m.GEO_CUBE_HEXA, 1, 2, 5, m.KIND_CD, 2)


@pytest.mark.parametrize("root,nref,nlev", [(1, 2, 3), (2, 1, 2)])
def test_stokes_setup_bit_exact(root, nref, nlev):
    """P2 (Dirichlet) / P1 (Neumann) numbering, combined [u1|u2|u3|p] structure
    and block prolongation of the Stokes hierarchy against the oracle"""
    from oracle import stokes as ost
    d = m.Discretization(m.GEO_CUBE_TETRA, root, nref, nlev, m.KIND_STOKES, 12)
    ref = ost.stokes_levels(root, nref, nlev)
    for l in range(nlev):
        r = ref[l]
        vi, pi = d.level_info(l, 0), d.level_info(l, 1)
        assert (vi["n_dofs"], vi["n_active"], pi["n_dofs"], pi["n_active"]) == (r.nu, r.nu_active, r.np_, r.np_)
        assert np.array_equal(d.dofmap(l, 0), r.udofmap)
        assert np.array_equal(d.dofmap(l, 1), r.pdofmap)
        rp, ci = d.structure(l)
        assert np.array_equal(rp, r.row_ptr) and np.array_equal(ci, r.cols)
        assert np.array_equal(d.cell_vertices(l).reshape(r.n_cells, -1), r.verts.reshape(r.n_cells, -1))
    rng = np.random.default_rng(3)
    for l in range(nlev - 1):
        rp, ci, v, nr, nc = d.prolongation(l)
        c, f = ref[l], ref[l + 1]
        assert (nr, nc) == (f.n, c.n)
        xc = rng.standard_normal(c.n)
        y = np.array([v[rp[i]:rp[i + 1]] @ xc[ci[rp[i]:rp[i + 1]]] for i in range(nr)])
        for b in range(4):
            lvc, lvf = _stokes_space(c, b), _stokes_space(f, b)
            ora = ocd.transfer(3, 12 if b < 3 else 11, lvc, lvf, xc[lvc.off:lvc.off + lvc.n_dofs], True)
            na = lvf.n_active
            assert np.allclose(y[lvf.off:lvf.off + na], ora[:na], rtol=0, atol=1e-13)


def test_stokes_workload_sizes():
    """3D Stokes workload: 24^3 cubes x 6 tetrahedra, three levels 6^3 / 12^3 / 24^3"""
    d = m.Discretization(m.GEO_CUBE_TETRA, 3, 3, 3, m.KIND_STOKES, 12)
    sizes = [(d.level_info(l, 0)["n_dofs"], d.level_info(l, 1)["n_dofs"], d.level_info(l)["n_cells"])
             for l in range(3)]
    assert sizes == [(2197, 343, 1296), (15625, 2197, 10368), (117649, 15625, 82944)]
    assert d.level_info(2)["nnz"] == 14183841


class _Sp:
    pass


def _stokes_space(lv, b):
    """one block of a Stokes level in the form oracle.cd.transfer takes"""
    z = _Sp()
    u = b < 3
    z.dofmap = lv.udofmap if u else lv.pdofmap
    z.verts, z.parent, z.n_cells = lv.verts, lv.parent, lv.n_cells
    z.nloc = 10 if u else 4
    z.n_dofs = lv.nu if u else lv.np_
    z.n_active = lv.nu_active if u else lv.np_
    z.off = b * lv.nu
    return z
