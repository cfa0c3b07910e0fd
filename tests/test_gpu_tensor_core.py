"""Tensor-core precision forms of the tangent (TF32 / BF16 operands, FP32
accumulation, tcgen05.mma) against the FP64 oracle.

Element matrices: per element, max |Ke_gpu - Ke_oracle| / max |Ke_oracle|.
The operands (8-node displacement bricks: the material-point values H and
the constant node-pair operator M; b-bar bricks: B and [D*]B; 20-node
bricks: Y = H n_b and the constant N_A) are rounded once to the input
format and the products accumulate in FP32, so the error scales with the
format's unit roundoff: TF32 (10 stored mantissa bits, u = 2^-11) stays
below 2e-3 and BF16 (7 bits, u = 2^-8) below 2e-2 of the element's
largest entry. The split forms (x = hi + lo in the input format, three
MMAs per product) carry about twice the bits: TF32X3 below 1e-5, BF16X3
below 2e-4. Every kernel projects the rigid translations out of each
element matrix after the accumulation, so Ke t stays at the FP32
rounding level.

Newton: the precision form changes only the tangent, never the residual,
so the solution at the 1e-8 relative residual is the FP64 one; the cost is
extra iterations (the tangent error sets the linear convergence rate).
"""
import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import loaded_state, make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Bilinear, Crystal, Model, Part, cube_mesh, mixed_mesh, random_orientations, \
    random_spans
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu

TOL = {abi.TANGENT_TF32: 2e-3, abi.TANGENT_BF16: 2e-2, abi.TANGENT_TF32X3: 1e-5, abi.TANGENT_BF16X3: 2e-4}
NAMES = {abi.TANGENT_TF32: "tf32", abi.TANGENT_BF16: "bf16", abi.TANGENT_TF32X3: "tf32x3",
         abi.TANGENT_BF16X3: "bf16x3"}
ALL = list(TOL)


def _engine(model, **kw):
    from warp3d_gb300.engine import Engine
    return Engine(model, **kw)


def _tangent_err(model, eng, ora, step, it, u, du):
    est_o = model.estiff_blocks()
    est_g = model.estiff_blocks()
    ora.tanstf(step, it, model.c, u, du, est_o)
    eng.tanstf(step, it, model.c, u, du, est_g)
    assert all(np.all(np.isfinite(g)) for g in est_g)
    return max(rel_err(g, o, axis=1) for g, o in zip(est_g, est_o))


def _loaded(model, nxyz, origins=None):
    ora, drv, du = loaded_state(model, nxyz, oracle.Oracle, steps=3, strain_per_step=0.0015,
                                shear_per_step=0.0 if origins is not None else 0.001, origins=origins)
    eng = _engine(model)
    eng.upload(ora.state)
    ifv = np.zeros(model.nodof)
    o2 = oracle.Oracle(model, state=ora.state.copy())
    assert o2.recover(4, 1, False, model.c, drv.u, du, ifv.copy())[0] == 0
    assert eng.recover(4, 1, False, model.c, drv.u, du, ifv)[0] == 0
    return eng, o2, drv.u, du


@pytest.fixture(scope="module")
def plastic_hex8():
    # ragged blocks: tiles of 5 elements leave partial tiles at block ends
    model, nxyz = make_model(n=5, jitter=0.1, spans=[64, 37, 1, 23])
    return (model,) + _loaded(model, nxyz)


@pytest.mark.parametrize("precision", ALL)
def test_tensor_core_tangent_plastic_state(plastic_hex8, precision):
    model, eng, ora, u, du = plastic_hex8
    eng.set_precision(precision)
    err = _tangent_err(model, eng, ora, 4, 1, u, du)
    eng.set_precision(abi.TANGENT_FP64)
    print(f"{NAMES[precision]} tangent rel err vs fp64 oracle {err:.2e}")
    assert err <= TOL[precision]


def _unpack(packed):
    """(span, 300) packed upper triangles -> (span, 24, 24) symmetric."""
    n = 24
    iu = np.triu_indices(n)
    # packed position of (i, j), i <= j: j (j + 1) / 2 + i
    pos = iu[1] * (iu[1] + 1) // 2 + iu[0]
    K = np.zeros((packed.shape[0], n, n))
    K[:, iu[0], iu[1]] = packed[:, pos]
    K[:, iu[1], iu[0]] = packed[:, pos]
    return K


@pytest.mark.parametrize("precision", ALL)
def test_tensor_core_tangent_keeps_the_rigid_translations(plastic_hex8, precision):
    """Ke t = 0 for the element's three rigid translations t. The kernel
    projects the translations out of every node-pair block after the
    accumulation (whose error has a mean along them), so what is left is
    the FP32 rounding of the projected entries."""
    model, eng, ora, u, du = plastic_hex8
    eng.set_precision(precision)
    est = model.estiff_blocks()
    eng.tanstf(4, 1, model.c, u, du, est)
    eng.set_precision(abi.TANGENT_FP64)
    worst = 0.0
    for blk in est:
        K = _unpack(blk)
        scale = np.max(np.abs(K), axis=(1, 2))
        for d in range(3):
            t = np.zeros(24)
            t[8 * d:8 * d + 8] = 1.0
            worst = max(worst, float(np.max(np.max(np.abs(K @ t), axis=1) / scale)))
    print(f"{NAMES[precision]} max |Ke t| / max |Ke| = {worst:.1e}")
    assert worst <= 1e-6


@pytest.fixture(scope="module")
def plastic_hex8_many_tiles():
    """20^3 elements in random blocks of 1..128: 562 tiles over the 152
    CTAs, so every CTA runs its pipeline over several tiles (the small
    models give each CTA about one). The state: one recovery from the
    virgin state over an affine increment (0.4% axial, 0.15% shear) with
    noise, which yields most of the mesh."""
    spans = random_spans(8000, np.random.Generator(np.random.PCG64(3)), lo=1, hi=128)
    model, _ = make_model(n=20, jitter=0.1, spans=spans)
    c = model.coords
    du = np.zeros(model.nodof)
    du[2::3] = 0.004 * c[:, 2]
    du[0::3] = 0.0015 * c[:, 2]
    du += np.random.Generator(np.random.PCG64(11)).normal(0.0, 2e-4, model.nodof)
    u = np.zeros(model.nodof)
    ora = oracle.Oracle(model)
    eng = _engine(model)
    ifv = np.zeros(model.nodof)
    st, info = ora.recover(2, 2, False, model.c, u, du, ifv.copy())
    assert st == 0 and info.plastic_work > 0.0
    assert eng.recover(2, 2, False, model.c, u, du, ifv)[0] == 0
    return model, eng, ora, u, du


@pytest.mark.parametrize("precision", ALL)
def test_tensor_core_tangent_several_tiles_per_cta(plastic_hex8_many_tiles, precision):
    model, eng, ora, u, du = plastic_hex8_many_tiles
    eng.set_precision(precision)
    err = _tangent_err(model, eng, ora, 2, 2, u, du)
    est = model.estiff_blocks()
    eng.tanstf(2, 2, model.c, u, du, est)
    eng.set_precision(abi.TANGENT_FP64)
    worst = 0.0
    for blk in est:
        K = _unpack(blk)
        scale = np.max(np.abs(K), axis=(1, 2))
        for d in range(3):
            t = np.zeros(24)
            t[8 * d:8 * d + 8] = 1.0
            worst = max(worst, float(np.max(np.max(np.abs(K @ t), axis=1) / scale)))
    print(f"{NAMES[precision]} 8000 elements: rel err {err:.2e}, max |Ke t| / max |Ke| = {worst:.1e}")
    assert err <= TOL[precision] and worst <= 1e-6


def test_tensor_core_wait_limit_zero_reports_efatal_without_a_fault(plastic_hex8):
    """A wait limit of 0: every tile gives up before its first MMA, Ke is
    NaN, w3g_tanstf returns W3G_EFATAL once; with the default limit the
    next call is correct again."""
    model, eng, ora, u, du = plastic_hex8
    for precision in (abi.TANGENT_TF32, abi.TANGENT_BF16X3):
        eng.set_precision(precision)
        eng.set_wait_limit(0)
        est = model.estiff_blocks()
        with pytest.raises(abi.W3GError) as ei:
            eng.tanstf(4, 1, model.c, u, du, est)
        assert ei.value.code == abi.EFATAL
        assert all(np.all(np.isnan(b)) for b in est)
        assert eng.check_finite() > 0
        eng.set_wait_limit(-1)
        assert _tangent_err(model, eng, ora, 4, 1, u, du) <= TOL[precision]
    eng.set_precision(abi.TANGENT_FP64)


@pytest.mark.parametrize("precision", ALL)
def test_tensor_core_tangent_linear_iteration_zero(plastic_hex8, precision):
    # iteration 0: no geometric term from the rotation update path, elastic D
    model, eng, ora, u, du = plastic_hex8
    eng.set_precision(precision)
    err = _tangent_err(model, eng, ora, 4, 0, u, du)
    eng.set_precision(abi.TANGENT_FP64)
    assert err <= TOL[precision]


def test_tensor_core_tangent_mixed_types():
    """8-node and 20-node bricks on the tensor cores, tetrahedra on the
    CUDA cores, in the same call."""
    rng = np.random.Generator(np.random.PCG64(11))
    coords, parts, origins = mixed_mesh(
        [(abi.ETYPE_L3DISOP, 3), (abi.ETYPE_Q3DISOP, 2), (abi.ETYPE_TET10, 2)], ny=2, nz=3, jitter=0.05, seed=11)
    plist = []
    for etype, inc in parts:
        spans = random_spans(inc.shape[0], rng, 1, 20)
        plist.append(Part(etype, inc, spans, [Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)] * len(spans)))
    model = Model(coords, parts=plist)
    eng, ora, u, du = _loaded(model, (3, 2, 3), origins=origins)
    for precision in ALL:
        eng.set_precision(precision)
        err = _tangent_err(model, eng, ora, 4, 1, u, du)
        print(f"mixed {NAMES[precision]} tangent rel err {err:.2e}")
        assert err <= TOL[precision]
        # 8-node and 20-node tensor-core kernels + the tetrahedra items
        assert eng.last_launch_count() == 3


def test_tensor_core_tangent_crystal_plasticity():
    coords, incid = cube_mesh(3, jitter=0.05)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(27, 7), block_spans=[20, 7])
    ora = oracle.Oracle(model)
    fixed, topz = uniaxial_bcs(model, (3, 3, 3))
    drv = NewtonDriver(model, ora, fixed, tol=1e-8, maxit=60, extrapolate=True)
    for s in range(1, 4):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.0005 * 3
        drv.step(s, imp)
    eng = _engine(model)
    eng.upload(ora.state)
    for precision in ALL:
        eng.set_precision(precision)
        err = _tangent_err(model, eng, ora, 3, 1, drv.u, np.zeros(model.nodof))
        print(f"mm10 {NAMES[precision]} tangent rel err {err:.2e}")
        assert err <= TOL[precision]


@pytest.mark.parametrize("precision", [abi.TANGENT_TF32, abi.TANGENT_TF32X3, abi.TANGENT_BF16X3])
def test_tensor_core_tangent_newton_reaches_fp64_solution(precision):
    n, nsteps = 6, 5
    coords, incid = cube_mesh(n, jitter=0.1)
    runs = []
    for prec in (abi.TANGENT_FP64, precision):
        model = Model(coords, incid)
        eng = _engine(model, precision=prec)
        fixed, topz = uniaxial_bcs(model, (n, n, n))
        drv = NewtonDriver(model, eng, fixed, tol=1e-8, maxit=60)
        for s in range(1, nsteps + 1):
            imp = np.zeros(model.nodof)
            imp[topz] = 0.01 * n / nsteps
            drv.step(s, imp)
        runs.append(drv)
    its = [[h[1] for h in d.history] for d in runs]
    print(f"newton iterations per step: fp64 {its[0]}, {NAMES[precision]} {its[1]}")
    assert max(h[2][-1] for h in runs[1].history) <= 1e-8
    assert rel_err(runs[1].u, runs[0].u) < 1e-7


def test_bf16_tangent_newton_rate_on_small_mesh():
    """Single-pass BF16 Ke (relative error ~3e-3) on the 6^3 bar: the
    Newton contraction per iteration is the tangent's error amplified by
    the global stiffness's condition number, which grows with the mesh;
    records the iteration counts reached within 60 iterations, or the
    residual where they stall, without asserting convergence."""
    n, nsteps = 6, 5
    coords, incid = cube_mesh(n, jitter=0.1)
    model = Model(coords, incid)
    eng = _engine(model, precision=abi.TANGENT_BF16)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    drv = NewtonDriver(model, eng, fixed, tol=1e-8, maxit=60)
    imp = np.zeros(model.nodof)
    imp[topz] = 0.01 * n / nsteps
    try:
        drv.step(1, imp)
        print("bf16 tangent: step 1 converged in", drv.history[-1][1], "iterations")
    except RuntimeError as exc:
        print("bf16 tangent: step 1 stalls:", str(exc)[:160])


def test_tensor_core_tangent_in_a_graph_replay_equals_direct_launch(plastic_hex8):
    """w3g_iteration_dev captures the tensor-core kernel in its CUDA graph;
    the replayed Ke equals the directly launched one bit for bit."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    model, eng, ora, u, du = plastic_hex8
    dev = torch.device("cuda", 0)
    tc, tu, tdu = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (model.c, u, du))
    tifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    cudart = C.CDLL("libcudart.so")

    def ke():
        p, n = eng.estiff_device()
        t = torch.empty(n, dtype=torch.float32, device=dev)
        assert cudart.cudaMemcpy(C.c_void_p(t.data_ptr()), C.c_void_p(p), C.c_size_t(4 * n), 3) == 0
        return t.cpu().numpy()

    for precision in (abi.TANGENT_TF32, abi.TANGENT_BF16X3):
        eng.set_precision(precision)
        eng.tanstf_dev(4, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), stream)
        torch.cuda.synchronize()
        direct = ke()
        for _ in range(2):
            eng.iteration_dev(4, 1, False, abi.ITER_TANGENT, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(),
                              tifv.data_ptr(), stream)
        torch.cuda.synchronize()
        assert np.array_equal(ke(), direct)
    eng.set_precision(abi.TANGENT_FP64)


# the 20-node bricks' tensor-core kernel: the single forms round the
# element's Y once (BF16 with the constant N_A split), the X3 forms split
# both operands: the 8-node bricks' bounds
TOL20 = dict(TOL)


@pytest.fixture(scope="module")
def plastic_hex20():
    rng = np.random.Generator(np.random.PCG64(21))
    coords, parts, origins = mixed_mesh([(abi.ETYPE_Q3DISOP, 3)], ny=2, nz=3, jitter=0.05, seed=21)
    plist = [Part(et, inc, random_spans(inc.shape[0], rng, 1, 9),
                  [Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)]) for et, inc in parts]
    model = Model(coords, parts=plist)
    return (model,) + _loaded(model, (3, 2, 3), origins=origins)


def _unpack20(packed):
    n = 60
    iu = np.triu_indices(n)
    pos = iu[1] * (iu[1] + 1) // 2 + iu[0]
    K = np.zeros((packed.shape[0], n, n))
    K[:, iu[0], iu[1]] = packed[:, pos]
    K[:, iu[1], iu[0]] = packed[:, pos]
    return K


@pytest.mark.parametrize("precision", ALL)
def test_tensor_core_tangent_hex20(plastic_hex20, precision):
    """20-node bricks (27 Gauss points, ragged blocks) on the tensor cores:
    every element matrix against the FP64 oracle, and the rigid
    translations (projected out in the epilogue) at the FP32 rounding
    level."""
    model, eng, ora, u, du = plastic_hex20
    eng.set_precision(precision)
    err = _tangent_err(model, eng, ora, 4, 1, u, du)
    assert eng.last_launch_count() == 1   # the 20-node tensor-core kernel alone
    est = model.estiff_blocks()
    eng.tanstf(4, 1, model.c, u, du, est)
    eng.set_precision(abi.TANGENT_FP64)
    worst = 0.0
    for blk in est:
        K = _unpack20(blk)
        scale = np.max(np.abs(K), axis=(1, 2))
        for d in range(3):
            t = np.zeros(60)
            t[20 * d:20 * d + 20] = 1.0
            worst = max(worst, float(np.max(np.max(np.abs(K @ t), axis=1) / scale)))
    print(f"hex20 {NAMES[precision]} tangent rel err {err:.2e}, max |Ke t| / max |Ke| = {worst:.1e}")
    assert err <= TOL20[precision]
    assert worst <= 1e-6


@pytest.fixture(scope="module")
def plastic_hex20_many_records():
    """14^3 20-node bricks in random blocks of 1..128: 361 records of up to
    8 elements over 152-304 CTAs, so CTAs cross records (the small model
    gives each CTA one). State: one recovery from the virgin state over an
    affine increment with noise (plastic)."""
    spans = random_spans(14 ** 3, np.random.Generator(np.random.PCG64(5)), lo=1, hi=128)
    model, _ = make_model(n=14, jitter=0.05, spans=spans, etype=abi.ETYPE_Q3DISOP)
    c = model.coords
    du = np.zeros(model.nodof)
    du[2::3] = 0.004 * c[:, 2]
    du[0::3] = 0.0015 * c[:, 2]
    du += np.random.Generator(np.random.PCG64(11)).normal(0.0, 2e-4, model.nodof)
    u = np.zeros(model.nodof)
    ora = oracle.Oracle(model)
    eng = _engine(model)
    ifv = np.zeros(model.nodof)
    st, info = ora.recover(2, 2, False, model.c, u, du, ifv.copy())
    assert st == 0 and info.plastic_work > 0.0
    assert eng.recover(2, 2, False, model.c, u, du, ifv)[0] == 0
    return model, eng, ora, u, du


@pytest.mark.parametrize("precision", ALL)
def test_tensor_core_tangent_hex20_several_records_per_cta(plastic_hex20_many_records, precision):
    model, eng, ora, u, du = plastic_hex20_many_records
    eng.set_precision(precision)
    err = _tangent_err(model, eng, ora, 2, 2, u, du)
    est = model.estiff_blocks()
    eng.tanstf(2, 2, model.c, u, du, est)
    eng.set_precision(abi.TANGENT_FP64)
    worst = 0.0
    for blk in est:
        K = _unpack20(blk)
        scale = np.max(np.abs(K), axis=(1, 2))
        for d in range(3):
            t = np.zeros(60)
            t[20 * d:20 * d + 20] = 1.0
            worst = max(worst, float(np.max(np.max(np.abs(K @ t), axis=1) / scale)))
    print(f"hex20 {NAMES[precision]} 2,744 elements: rel err {err:.2e}, max |Ke t| / max |Ke| = {worst:.1e}")
    assert err <= TOL20[precision] and worst <= 1e-6


def test_tensor_core_hex20_wait_limit_zero_reports_efatal(plastic_hex20):
    model, eng, ora, u, du = plastic_hex20
    eng.set_precision(abi.TANGENT_TF32)
    eng.set_wait_limit(0)
    est = model.estiff_blocks()
    with pytest.raises(abi.W3GError) as exc:
        eng.tanstf(4, 1, model.c, u, du, est)
    assert exc.value.code == abi.EFATAL
    assert all(np.all(np.isnan(b)) for b in est)
    # the context stays usable: the next call with the default limit is right
    eng.set_wait_limit(-1)
    assert _tangent_err(model, eng, ora, 4, 1, u, du) <= TOL20[abi.TANGENT_TF32]
    eng.set_precision(abi.TANGENT_FP64)
