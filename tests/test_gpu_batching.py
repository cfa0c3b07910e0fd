"""Batching form: per-type launches vs the persistent work-queue kernels,
the CUDA-graph iteration and the autotuner, on a model that mixes 8-node
bricks, 20-node bricks and 10-node tetrahedra in blocks of uneven size.

The schedule only reorders work, so every output must be bitwise equal
across schedules and between direct launches and graph replays; a Newton
solution run entirely through graph replays with the persistent kernels
and the FP32 tangent must reach the FP64 solution to the 1e-8 relative
global residual.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests.conftest import rel_err
from tests.helpers import loaded_state
from tests.test_gpu_parity_types import _mixed_model
from warp3d_gb300 import abi
from warp3d_gb300.newton import NewtonDriver, uniaxial_bcs

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _engine(model, **kw):
    from warp3d_gb300.engine import Engine
    return Engine(model, **kw)


@pytest.fixture(scope="module")
def mixed_case():
    model, origins = _mixed_model()
    ora, drv, du = loaded_state(model, (3, 2, 3), oracle.Oracle, steps=3, strain_per_step=0.0015, origins=origins)
    return model, ora.state, drv.u.copy(), du


class _Dev:
    def __init__(self, model, u, du):
        dev = torch.device("cuda", 0)
        self.c = torch.from_numpy(model.c).to(dev)
        self.u = torch.from_numpy(np.asarray(u)).to(dev)
        self.du = torch.from_numpy(np.asarray(du)).to(dev)
        self.ifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)

    def ptrs(self):
        return self.c.data_ptr(), self.u.data_ptr(), self.du.data_ptr(), self.ifv.data_ptr()


def _estiff(eng, fp32):
    ptr, n = eng.estiff_device()
    t = torch.empty(n, dtype=torch.float32 if fp32 else torch.float64, device="cuda")
    cudart = C.CDLL("libcudart.so")
    assert cudart.cudaMemcpy(C.c_void_p(t.data_ptr()), C.c_void_p(ptr), C.c_size_t(t.element_size() * n), 3) == 0
    return t.cpu().numpy()


def _outputs(model, eng, dev, fp32):
    torch.cuda.synchronize()
    st, info = eng.recover_info()
    got = model.new_state()
    eng.download(got)
    arrays = {n: np.concatenate([a.reshape(-1) for a in getattr(got, n)])
              for n in ("urcs_n1", "eps_n1", "rot_n1", "history1", "cep", "einfvec", "element_vol")}
    arrays["ifv"] = dev.ifv.cpu().numpy()
    arrays["energy"] = np.array([info.internal_energy, info.plastic_work, info.sum_ifv])
    arrays["estiff"] = _estiff(eng, fp32)
    return arrays


def _run_direct(model, state, u, du, sched, fp32, step=4, it=1):
    eng = _engine(model, precision=abi.TANGENT_FP32 if fp32 else abi.TANGENT_FP64)
    eng.upload(state)
    if sched is not None:
        eng.set_schedule(**sched)
    dev = _Dev(model, u, du)
    c, uu, d, f = dev.ptrs()
    stream = torch.cuda.current_stream().cuda_stream
    eng.recover_dev(step, it, False, c, uu, d, f, stream)
    eng.tanstf_dev(step, it, c, uu, d, stream)
    return _outputs(model, eng, dev, fp32), eng


SCHEDULES = [
    dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_HEAVY_FIRST),
    dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_BLOCKS, recover_ctas_per_sm=1, tangent_ctas_per_sm=1,
         recover_grain=3, tangent_grain=5),
    dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_HEAVY_FIRST, recover_ctas_per_sm=2, tangent_grain=2),
]


@pytest.mark.parametrize("fp32", [False, True], ids=["fp64", "fp32"])
def test_persistent_schedules_match_per_type_bitwise(mixed_case, fp32):
    model, state, u, du = mixed_case
    ref, eng = _run_direct(model, state, u, du, None, fp32)
    assert eng.schedule()["mode"] == abi.SCHED_PER_TYPE
    for sc in SCHEDULES:
        got, eng = _run_direct(model, state, u, du, sc, fp32)
        assert eng.last_launch_count() == 1   # the tangent call: one persistent launch
        for k in ref:
            assert np.array_equal(got[k], ref[k]), (sc, k)


def test_graph_iteration_matches_direct_calls(mixed_case):
    model, state, u, du = mixed_case
    for sched in (None, SCHEDULES[0]):
        ref, _ = _run_direct(model, state, u, du, sched, True, step=4, it=0)
        ref1, _ = _run_direct(model, state, u, du, sched, True, step=4, it=2)
        eng = _engine(model, precision=abi.TANGENT_FP32)
        eng.upload(state)
        if sched is not None:
            eng.set_schedule(**sched)
        dev = _Dev(model, u, du)
        stream = torch.cuda.current_stream().cuda_stream
        both = abi.ITER_RECOVER | abi.ITER_TANGENT
        # iteration 0, then a replay of the same graph with iteration 2
        eng.iteration_dev(4, 0, False, both, *dev.ptrs(), stream)
        got = _outputs(model, eng, dev, True)
        for k in ref:
            assert np.array_equal(got[k], ref[k]), (sched, k)
        eng.iteration_dev(4, 2, False, both, *dev.ptrs(), stream)
        got = _outputs(model, eng, dev, True)
        for k in ref1:
            assert np.array_equal(got[k], ref1[k]), (sched, k)
        per = 3 if sched is None else 1
        assert eng.last_launch_count() == 1 + (5 + per) + per


def test_autotune_picks_valid_schedule_and_leaves_one_iteration(mixed_case):
    model, state, u, du = mixed_case
    ref, _ = _run_direct(model, state, u, du, None, True, step=4, it=1)
    eng = _engine(model, precision=abi.TANGENT_FP32)
    eng.upload(state)
    dev = _Dev(model, u, du)
    stream = torch.cuda.current_stream().cuda_stream
    sched, ms = eng.autotune(4, 1, False, *dev.ptrs(), stream, reps=2)
    print("autotuned", sched, f"{ms:.3f} ms")
    assert sched["mode"] in (abi.SCHED_PER_TYPE, abi.SCHED_PERSISTENT) and ms > 0
    assert eng.schedule() == sched
    got = _outputs(model, eng, dev, True)
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k


class GraphEngine:
    """The Engine.recover / Engine.tanstf interface the Newton driver uses,
    run through w3g_iteration_dev graph replays on device buffers."""

    def __init__(self, model, precision, sched):
        self.model = model
        self.fp32 = precision == abi.TANGENT_FP32
        self.eng = _engine(model, precision=precision)
        if sched is not None:
            self.eng.set_schedule(**sched)
        self.dev = _Dev(model, np.zeros(model.nodof), np.zeros(model.nodof))
        self.stream = torch.cuda.current_stream().cuda_stream

    def _load(self, c, u, du):
        self.dev.c.copy_(torch.from_numpy(c))
        self.dev.u.copy_(torch.from_numpy(u))
        self.dev.du.copy_(torch.from_numpy(du))

    def recover(self, step, it, extrap, c, u, du, ifv):
        self._load(c, u, du)
        self.eng.iteration_dev(step, it, extrap, abi.ITER_RECOVER, *self.dev.ptrs(), self.stream)
        torch.cuda.synchronize()
        st, info = self.eng.recover_info()
        ifv[:] = self.dev.ifv.cpu().numpy()
        return st, info

    def tanstf(self, step, it, c, u, du, estiff_blocks):
        self._load(c, u, du)
        self.eng.iteration_dev(step, it, False, abi.ITER_TANGENT, *self.dev.ptrs(), self.stream)
        torch.cuda.synchronize()
        k = _estiff(self.eng, self.fp32).astype(np.float64)
        off = 0
        for b in estiff_blocks:
            b[:] = k[off:off + b.size].reshape(b.shape)
            off += b.size

    def update(self):
        self.eng.update()


def test_batched_mixed_precision_newton_reaches_fp64_solution():
    model, origins = _mixed_model()

    def run(engine):
        fixed, topz = uniaxial_bcs(model, (3, 2, 3), origins=origins)
        drv = NewtonDriver(model, engine, fixed, tol=1e-8)
        for s in range(1, 4):
            imp = np.zeros(model.nodof)
            imp[topz] = 0.0015 * 3
            drv.step(s, imp)
        return drv

    d64 = run(_engine(model))
    dmx = run(GraphEngine(model, abi.TANGENT_FP32, SCHEDULES[0]))
    its64 = [h[1] for h in d64.history]
    itsmx = [h[1] for h in dmx.history]
    print("newton iterations per step: fp64 per-type", its64, "fp32 persistent graph", itsmx)
    assert max(h[2][-1] for h in dmx.history) <= 1e-8
    assert rel_err(dmx.u, d64.u) < 1e-7
