"""The sliced-ELL SpMV kernel (context options fp32_sliced_spmv and
fp64_sliced_spmv) against the FP64 oracle, against the row-group kernels, and
inside the multigrid (Jacobi sweeps, defects and restriction run on the sliced
copies). The cases have more than 16 entries per row on their finest level,
the matrices that get a sliced copy.

Tolerances: FP32 SpMV within 2e-6 of sum_j |a_ij x_j| (FP32 rounding of about
60 products per row); shapes with the same lanes per row sum in the same order
and must agree bit for bit."""
import numpy as np
import pytest

import mymoonmd_gb300 as m
from oracle import cd as ocd

from test_gpu_parity import CASES, make_pair, mg_db, rel

pytestmark = pytest.mark.gpu

SHAPES = [140, 141, 180, 240, 241, 280, 440, 441, 480, 481, 840, 841, 881]
DEFAULT = 481


@pytest.fixture
def sliced(ctx):
    """sets the shape for one test and puts the library default back"""
    def set_shape(shape):
        ctx.set_option("fp32_sliced_spmv", shape)
    yield set_shape
    ctx.set_option("fp32_sliced_spmv", DEFAULT)


def fp32_spmv(ctx, A, x):
    y = m.DeviceVector(ctx, x.size, np.float32)
    A.apply_f32(m.DeviceVector.from_numpy(ctx, x.astype(np.float32)), y)
    return y.numpy()


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("case", ["q2_3d", "q2_3d_root3"])
def test_sliced_spmv_matches_fp64_within_fp32_rounding(ctx, sliced, case, shape):
    disc, prob, ora = make_pair(ctx, case, mg_db(CASES[case][3]))
    A = prob.matrix(-1)
    sliced(shape)
    A.make_fp32()  # lays out the sliced copy for the shape's lanes per row
    lv = ora.finest
    x = np.random.default_rng(4).standard_normal(lv.n_dofs)
    y = fp32_spmv(ctx, A, x)
    ref = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x, np.zeros(lv.n_dofs), 1.0)
    scale = ocd.apply_scaled_add(lv.row_ptr, lv.cols, np.abs(ora.vals[-1]), ora.active(), np.abs(x),
                                 np.zeros(lv.n_dofs), 1.0)
    assert np.all(np.abs(y - ref) <= 2e-6 * scale + 1e-30)


def test_sliced_shapes_with_equal_lanes_give_equal_bits(ctx, sliced):
    """U (steps in flight) and the load pipelining change no summation order:
    the SpMV and a whole mixed multigrid application are identical for all
    shapes with the same lanes per row"""
    disc, prob, ora = make_pair(ctx, "q2_3d", mg_db(3, precision="mixed"))
    prob.solve()
    A = prob.matrix(-1)
    n = ora.finest.n_dofs
    rng = np.random.default_rng(9)
    x = rng.standard_normal(n)
    z = m.DeviceVector.from_numpy(ctx, rng.standard_normal(n))
    out = {}
    for shape in SHAPES:
        sliced(shape)
        prob.reset_solution()
        prob.assemble()
        prob.solve()  # the multigrid update lays out every level's sliced copies
        r = m.DeviceVector(ctx, n)
        prob.solver().apply_preconditioner(z, r)
        out[shape] = (fp32_spmv(ctx, A, x), r.numpy())
    for lanes in (1, 2, 4, 8):
        group = [s for s in SHAPES if s // 100 == lanes]
        for s in group[1:]:
            assert np.array_equal(out[group[0]][0], out[s][0]), (group[0], s)
            assert np.array_equal(out[group[0]][1], out[s][1]), (group[0], s)
    # different lanes per row sum in different orders: the layouts are in use
    assert not np.array_equal(out[140][0], out[440][0])
    assert not np.array_equal(out[140][1], out[440][1])


@pytest.mark.parametrize("shape", [0, 180, 241, 481, 841])
def test_mixed_precision_with_each_fp32_kernel_reaches_fp64_target(ctx, sliced, shape):
    """the mixed form on the row-group kernel (0) and on sliced shapes: the
    1e-8 FP64 residual reduction and the FP64 oracle solution within 1e-7"""
    sliced(shape)
    db = mg_db(3, restart=30, reduction=1e-8, precision="mixed")
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    it, res, init = prob.last_info()
    assert res <= 1e-8 * init and it < 200
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, *_ = ora.solve("fgmres", 0.0, 1e-8, 200, 0, 30)
    assert rel(prob.solution(), sol) <= 1e-7


@pytest.mark.parametrize("coarse_residual", [0.0, 1.0])
def test_sliced_kernel_in_iterative_coarse_loop(ctx, sliced, coarse_residual):
    """FP32 Jacobi on the coarsest level with the device-side stop (the sliced
    kernel's guarded no-op copies the iterate): the multigrid application agrees
    with the row-group kernel's within FP32 rounding"""
    out = {}
    for shape in (0, DEFAULT):
        sliced(shape)
        db = mg_db(3, precision="mixed")
        db["multigrid_smoother_coarse"] = "jacobi"
        db["multigrid_coarse_max_n_iterations"] = 10
        db["multigrid_coarse_residual"] = coarse_residual
        disc, prob, ora = make_pair(ctx, "q2_3d", db)
        prob.solve()
        z = np.random.default_rng(5).standard_normal(ora.finest.n_dofs)
        r = m.DeviceVector(ctx, z.size)
        prob.solver().apply_preconditioner(m.DeviceVector.from_numpy(ctx, z), r)
        out[shape] = r.numpy()
        prob.close()
    assert rel(out[DEFAULT], out[0]) <= 1e-4


SHAPES64 = [441, 481, 841]
DEFAULT64 = 441


@pytest.fixture
def sliced64(ctx):
    """sets the FP64 shape for one test and puts the library default back"""
    def set_shape(shape):
        ctx.set_option("fp64_sliced_spmv", shape)
    yield set_shape
    ctx.set_option("fp64_sliced_spmv", DEFAULT64)


@pytest.mark.parametrize("shape", SHAPES64)
@pytest.mark.parametrize("case", ["q2_3d", "q2_3d_root3"])
def test_fp64_sliced_spmv_matches_oracle(ctx, sliced64, case, shape):
    """the FP64 sliced copy (laid out by the solver's update) gives
    apply_scaled_add within 1e-13 of sum_j |a_ij x_j| of the oracle. With 4
    lanes per row it sums each row in the order of the FP64 row-group kernel
    (4 lanes, entries j = lane mod 4, pairs combined (0+2)+(1+3)): the same
    bits; with 8 lanes the order differs (the sliced kernel is in use)"""
    sliced64(shape)
    disc, prob, ora = make_pair(ctx, case, mg_db(CASES[case][3]))
    prob.solve()  # update: the FP64 sliced copies of every level
    A = prob.matrix(-1)
    lv = ora.finest
    rng = np.random.default_rng(3)
    x = rng.standard_normal(lv.n_dofs)
    y0 = rng.standard_normal(lv.n_dofs)
    out = {}
    for s in (shape, 0):
        sliced64(s)
        xd, yd = m.DeviceVector.from_numpy(ctx, x), m.DeviceVector.from_numpy(ctx, y0)
        A.apply_scaled_add(xd, yd, -0.7)
        out[s] = yd.numpy()
    ref = ocd.apply_scaled_add(lv.row_ptr, lv.cols, ora.vals[-1], ora.active(), x, y0, -0.7)
    scale = ocd.apply_scaled_add(lv.row_ptr, lv.cols, np.abs(ora.vals[-1]), ora.active(), np.abs(x),
                                 np.abs(y0), 0.7)
    assert np.all(np.abs(out[shape] - ref) <= 1e-13 * scale)
    if shape // 100 == 4:
        assert np.array_equal(out[shape], out[0])
    else:
        assert not np.array_equal(out[shape], out[0])


@pytest.mark.parametrize("shape", [0, 441, 841])
def test_fp64_form_with_each_kernel_matches_oracle(ctx, sliced64, shape):
    """the FP64 form (Krylov SpMV, Jacobi sweeps, defects, restriction on the
    FP64 sliced copies): final solution within 1e-10 of the oracle's, FGMRES
    iteration counts within one"""
    sliced64(shape)
    db = mg_db(3, restart=20, reduction=1e-10)
    disc, prob, ora = make_pair(ctx, "q2_3d", db)
    prob.solve()
    it, res, init = prob.last_info()
    ora.build_mg(2, 2, 0.8, 1.0, "V")
    sol, oit, ores, ohist, st = ora.solve("fgmres", 0.0, 1e-10, 200, 0, 20)
    assert abs(it - oit) <= 1
    assert rel(prob.solution(), sol) <= 1e-10
