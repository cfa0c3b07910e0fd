"""Device assembly of the global stiffness, the device PCG solve and the
device Newton loop, against the host path (SciPy assembly and sparse
direct solve, newton.py).

Assembly: the device CSR equals the host COO->CSR sum of the same element
matrices to 1e-14 relative (the two sum each coefficient's contributions
in different orders); two assemblies are bitwise equal. PCG: the solution
of K_ff x = b matches spsolve to 1e-9 at rtol 1e-12; two solves are
bitwise equal. Newton: the device loop takes the host loop's iteration
counts and reaches its displacements to 1e-8.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from tests.conftest import rel_err
from tests.helpers import make_model
from warp3d_gb300 import abi
from warp3d_gb300.model import Bilinear, Model, Part, cube_mesh, mixed_mesh, random_spans
from warp3d_gb300.newton import Assembler, NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu


def _engine(model, **kw):
    from warp3d_gb300.engine import Engine
    return Engine(model, **kw)


def _mixed_model(seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    coords, parts, origins = mixed_mesh(
        [(abi.ETYPE_L3DISOP, 3), (abi.ETYPE_Q3DISOP, 2), (abi.ETYPE_TET10, 2)], ny=2, nz=2, jitter=0.05, seed=seed)
    plist = [Part(et, inc, random_spans(inc.shape[0], rng, 1, 9), [Bilinear.from_hprime(200000.0, 0.3, 400.0,
                                                                                          2000.0)])
             for et, inc in parts]
    return Model(coords, parts=plist)


def _state_after_tangent(model, precision):
    from warp3d_gb300.solver import DeviceCsr
    eng = _engine(model, precision=precision)
    rng = np.random.default_rng(2)
    du = rng.normal(0.0, 1e-3, model.nodof)
    u = np.zeros(model.nodof)
    ifv = np.zeros(model.nodof)
    assert eng.recover(1, 1, False, model.c, u, du, ifv)[0] == 0
    est = model.estiff_blocks()
    eng.tanstf(1, 1, model.c, u, du, est)
    csr = DeviceCsr(eng)
    return eng, csr, est


@pytest.mark.parametrize("kind", ["hex8", "mixed"])
@pytest.mark.parametrize("precision", [abi.TANGENT_FP64, abi.TANGENT_FP32])
def test_device_assembly_matches_host(kind, precision):
    model = make_model(n=4, jitter=0.1, spans=[30, 34])[0] if kind == "hex8" else _mixed_model()
    eng, csr, est = _state_after_tangent(model, precision)
    csr.assemble()
    K_dev = csr.to_scipy()
    K_host = Assembler(model).assemble(est)
    assert K_dev.shape == K_host.shape
    diff = abs(K_dev - K_host).max()
    print(f"{kind} precision {precision}: nnz {K_dev.nnz} vs {K_host.nnz}, max |dK| / max |K| "
          f"{diff / abs(K_host).max():.2e}")
    assert K_dev.nnz == K_host.nnz
    assert diff <= 1e-14 * abs(K_host).max()
    csr.assemble()
    K2 = csr.to_scipy()
    assert np.array_equal(K2.data, K_dev.data)


def test_device_pcg_matches_direct_solve():
    torch = pytest.importorskip("torch")
    model, nxyz = make_model(n=5, jitter=0.1, spans=[60, 65])
    eng, csr, est = _state_after_tangent(model, abi.TANGENT_FP64)
    csr.assemble()
    fixed, _ = uniaxial_bcs(model, nxyz)
    free = np.setdiff1d(np.arange(model.nodof), fixed)
    rng = np.random.default_rng(9)
    b = rng.normal(size=model.nodof)
    dev = torch.device("cuda", 0)
    tb = torch.from_numpy(b).to(dev)
    tx = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    mask = torch.zeros(model.nodof, dtype=torch.uint8, device=dev)
    mask[torch.from_numpy(fixed).to(dev)] = 1
    st, its, rel = csr.pcg(mask.data_ptr(), tb.data_ptr(), -2.0, tx.data_ptr(), 1e-12, 20000)
    assert st == 0 and rel <= 1e-12
    x = tx.cpu().numpy()
    K = Assembler(model).assemble(est).tocsr()
    ref = spla.spsolve(K[free][:, free].tocsc(), -2.0 * b[free])
    print(f"pcg: {its} iterations, relres {rel:.2e}, rel err vs spsolve {rel_err(x[free], ref):.2e}")
    assert rel_err(x[free], ref) < 1e-9
    assert np.all(x[fixed] == 0.0)
    tx2 = torch.zeros_like(tx)
    st2, its2, _ = csr.pcg(mask.data_ptr(), tb.data_ptr(), -2.0, tx2.data_ptr(), 1e-12, 20000)
    assert st2 == 0 and its2 == its
    assert torch.equal(tx, tx2)
    # iteration limit
    st3, its3, rel3 = csr.pcg(mask.data_ptr(), tb.data_ptr(), 1.0, tx2.data_ptr(), 1e-12, 5)
    assert st3 == abi.PCG_MAXIT and rel3 > 1e-12
    # the row kernels with the diagonal preconditioner reach the same solution
    assert csr.set_node_blocks(False) is False
    tx3 = torch.zeros_like(tx)
    st4, its4, rel4 = csr.pcg(mask.data_ptr(), tb.data_ptr(), -2.0, tx3.data_ptr(), 1e-12, 20000)
    print(f"pcg, row kernels and diagonal preconditioner: {its4} iterations (node blocks: {its})")
    assert st4 == 0 and rel_err(tx3.cpu().numpy()[free], ref) < 1e-9
    assert csr.set_node_blocks(True) is True
    # norms on the device
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    csr.residual_norms(tb.data_ptr(), mask.data_ptr(), out.data_ptr())
    nf, na = out.cpu().numpy()
    assert abs(nf - np.dot(b[free], b[free])) <= 1e-13 * nf
    assert abs(na - np.dot(b, b)) <= 1e-13 * na


def test_device_newton_matches_host_newton():
    from warp3d_gb300.solver import DeviceNewtonDriver
    n, nsteps = 5, 4
    coords, incid = cube_mesh(n, jitter=0.1)
    runs = []
    for drv_cls in (NewtonDriver, DeviceNewtonDriver):
        model = Model(coords, incid)
        eng = _engine(model)
        fixed, topz = uniaxial_bcs(model, (n, n, n))
        kw = {"lin_rtol": 1e-12} if drv_cls is DeviceNewtonDriver else {}
        drv = drv_cls(model, eng, fixed, tol=1e-8, **kw)
        for s in range(1, nsteps + 1):
            imp = np.zeros(model.nodof)
            imp[topz] = 0.01 * n / nsteps
            drv.step(s, imp)
        runs.append(drv)
    its = [[h[1] for h in d.history] for d in runs]
    print("newton iterations host / device", its, "pcg iterations", runs[1].lin_history)
    assert its[0] == its[1]
    assert rel_err(runs[1].u, runs[0].u) < 1e-8


def test_device_newton_adaptive_subdivision():
    """A first step too large for Newton from the linear predictor is cut
    into sub-increments that converge; every increment's fraction is
    recorded and the fractions of a step sum to one."""
    from warp3d_gb300.solver import DeviceNewtonDriver
    n = 10
    coords, incid = cube_mesh(n, jitter=0.1)
    model = Model(coords, incid)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    drv = DeviceNewtonDriver(model, _engine(model), fixed, tol=1e-8, maxit=12, lin_rtol=1e-11, extrapolate=True,
                             adaptive=True, adaptive_step1=True)
    for s in (1, 2):
        imp = np.zeros(model.nodof)
        imp[topz] = 0.02 * n
        drv.step(s, imp)
    print("increments", len(drv.history), "cuts", drv.cuts, "fractions", drv.fractions,
          "newton", [h[1] for h in drv.history])
    assert all(h[2][-1] <= 1e-8 for h in drv.history)
    steps = [h[0] for h in drv.history]
    for s in (1, 2):
        assert abs(sum(f for f, t in zip(drv.fractions, steps) if t == s) - 1.0) < 1e-12


@pytest.mark.parametrize("kind", ["hex8", "mixed"])
@pytest.mark.parametrize("forcing", ["fixed", "ew"])
def test_newton_iteration_graph_equals_step_by_step(kind, forcing):
    """One graph per Newton iteration (w3g_newton_iteration_dev: the PCG as
    a device-side conditional loop, du += d, recovery, tangent, assembly,
    norms) against the same loop driven call by call: the same kernels in
    the same order, so iteration counts, PCG counts and displacements are
    bitwise equal; with the FP32 tangent too (the mixed model)."""
    from warp3d_gb300.solver import DeviceNewtonDriver
    if kind == "hex8":
        n = 5
        coords, incid = cube_mesh(n, jitter=0.1)
        mk = lambda: Model(coords, incid)
        nxyz, origins, strain, prec = (n, n, n), None, 0.01, abi.TANGENT_FP64
    else:
        coords, parts, origins = mixed_mesh(
            [(abi.ETYPE_L3DISOP, 3), (abi.ETYPE_Q3DISOP, 2), (abi.ETYPE_TET10, 2)], ny=2, nz=2, jitter=0.05, seed=5)
        rng = np.random.Generator(np.random.PCG64(5))
        spans = [random_spans(inc.shape[0], rng, 1, 9) for _, inc in parts]
        mk = lambda: Model(coords, parts=[Part(et, inc, sp, [Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)])
                                          for (et, inc), sp in zip(parts, spans)])
        nxyz, strain, prec = (3, 2, 2), 0.004, abi.TANGENT_FP32
    runs = []
    for graph in (False, True):
        model = mk()
        eng = _engine(model)
        eng.set_precision(prec)
        fixed, topz = uniaxial_bcs(model, nxyz, origins=origins)
        drv = DeviceNewtonDriver(model, eng, fixed, tol=1e-8, maxit=40, lin_rtol=1e-10, extrapolate=True,
                                 forcing=forcing, eta_max=1e-3, graph=graph)
        for s in range(1, 4):
            imp = np.zeros(model.nodof)
            imp[topz] = strain * nxyz[2] / 3
            drv.step(s, imp)
        runs.append((drv, eng))
    (a, _), (b, eb) = runs
    print("newton", [h[1] for h in a.history], "pcg", [l for _, l in a.lin_history])
    assert [h[1] for h in a.history] == [h[1] for h in b.history]
    assert [l for _, l in a.lin_history] == [l for _, l in b.lin_history]
    assert np.array_equal(a.u, b.u)
