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
