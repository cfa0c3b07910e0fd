#!/usr/bin/env python
"""Newton-iteration element throughput of the element-block hot path.

Workload: the plain FP64 GPU path at scale -- a 64x64x64 mesh of 8-node
bricks (262,144 elements, 2,097,152 Gauss points), interior nodes jittered
U(-0.1, 0.1) h (PCG64(12345)), mm01 bilinear Mises (E = 200 GPa,
nu = 0.3, yield 400 MPa, H' = 2 GPa, isotropic), element blocks of 128.
Synthetic data: the state is set by one load step to 1% uniaxial strain
(every Gauss point plastic); each timed step is one Newton iteration of
the element work -- one tangent (tanstf) plus one strain/stress/internal
force recovery (drive_eps_sig_internal_forces) -- on a perturbed
increment. Inputs (~3 GB of element state per iteration) exceed the
129 MB L2, so no flush is needed between steps.

metric: elements per second per Newton iteration
        = n_elements / (t_tangent + t_recovery).
value:  plain FP64 form, inputs resident in HBM (device-pointer C-ABI).
mixed:  the same iteration with the FP32 tangent (recovery stays FP64).
e2e:    the host-array C-ABI calls a Fortran caller makes (w3g_tanstf
        with host estiff blocks + w3g_recover with host ifv), all
        host<->device copies inside the timed region.
batched: the batching-form workload -- about 1M elements in blocks of
        random size uniform in [16, 128] (PCG64), 60% 8-node bricks, 25%
        20-node bricks, 15% 10-node tetrahedra (three bars of one type
        each, 64 x 64 cells in cross-section, jitter U(-0.05, 0.05) h),
        mm01 with yield per block U(250, 550) MPa; one Newton iteration
        per step through w3g_iteration_dev (graph replay), FP64 and with
        the FP32 tangent, each under the schedule w3g_autotune picks, next
        to the per-type launches without a graph.
formulations: the same mesh, state and increment with WARP3D's default
        l3disop formulation (b-bar mean dilatation, finite strain) and with
        the small-displacement b-bar brick of its published example model;
        FP64, FP32 and TF32 tangents.
crystal: mm10 crystal plasticity -- 32^3 8-node bricks (32,768 elements,
        262,144 Gauss points), one fcc crystal per Gauss point with Euler
        angles uniform on SO(3) (PCG64), Voce hardening (tau_y 90, tau_v
        200, theta_0 500 MPa, rate exponent 20); the state after 1%
        homogeneous tension in 10 steps; one Newton iteration of element
        work per step (graph replay), FP64 and with the FP32 tangent, the
        local Newton iteration counts per Gauss point, the work queue
        sorted by the previous counts vs in natural order, and the oracle
        on a bounded sample of the same blocks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton-iteration element throughput (elem/s) FP64 vs mixed @ equal residual"
UNIT = "elem/s"

# Algorithmic FP64 work per hex8 element per call, in flops (FMA = 2,
# add/mul = 1): the minimal counts of the quantities computed, per GP:
#   tangent  [J] 144, det/inverse 50, shape gradients 120, [D] scale 21,
#            [q] 54, {T} = [q]{t} 66, [q][D][q]^T lower triangle 627,
#            Q-bar 30, {T}w 6, D*B_b 720, {T}g_b 120,
#            B^T(D*B) upper triangle (900 multiply-adds) 1800, G^T T G 288
#            = 4046 flop/GP
#   recovery theta at n+1 and n+1/2 in reference order 360, det[F] 34,
#            2 polar decompositions 400 (plus per decomposition: atan2,
#            sin, cos, 5 sqrt, 1 division), d = sym(dDu/dX Fh^-1) 220,
#            unrotation 81, mm01 + cnst1 250, energy 12, Cauchy rotation
#            75, P = T F^-T 84, element forces 120, GP sums 21
#            = 1657 flop/GP
TANGENT_FLOP_PER_ELEM = 8 * 4046
RECOVER_FLOP_PER_ELEM = 8 * 1657
# the reference's dense operation counts (B as a full 6 x totdof matrix),
# reported beside ours in the JSON
TANGENT_FLOP_PER_ELEM_REFDENSE = 52992
RECOVER_FLOP_PER_ELEM_REFDENSE = 12000
# compulsory HBM bytes per element (FP64): tangent reads cep 21*8, coords
# 24, rot+urcs 18*8 per GP and writes Ke 300; recovery reads coordinates,
# u, du and the state at n (2,240 B) and writes the state at n+1, cep, R
# and the element forces (3,776 B).
TANGENT_BYTES_PER_ELEM = 8 * (21 * 8 + 24 + 48 + 18 * 8 + 300)
TANGENT32_BYTES_PER_ELEM = TANGENT_BYTES_PER_ELEM - 4 * 300
RECOVER_BYTES_PER_ELEM = 6016

# precision forms of the tangent on the tensor cores, and the one the
# headline "mixed" figure reports
TC_FORMS = (("tf32", 2), ("bf16", 3), ("tf32x3", 4), ("bf16x3", 5))
HEADLINE_FORM = "tf32"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=64, help="elements per cube edge")
    ap.add_argument("--cpu-sample-blocks", type=int, default=1024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-elems", type=int, default=1_000_000, help="target elements of the batched workload")
    ap.add_argument("--no-crystal", action="store_true")
    ap.add_argument("--crystal-n", type=int, default=32, help="elements per cube edge of the mm10 workload")
    ap.add_argument("--no-solver", action="store_true", help="skip the device assembly / PCG measurement")
    ap.add_argument("--no-formulations", action="store_true", help="skip the b-bar / small-displacement lines")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks on sampled blocks")
    ap.add_argument("--precision-study", action="store_true",
                    help="instead of the bench line: Newton solves of the cube under every tangent precision form")
    ap.add_argument("--study-steps", type=int, default=20)
    ap.add_argument("--study-strain", type=float, default=0.02)
    ap.add_argument("--study-forms", default="fp64,fp32,tf32,bf16,tf32x3,bf16x3")
    ap.add_argument("--study-maxit", type=int, default=25)
    ap.add_argument("--study-forcing", default="fixed", choices=["fixed", "ew"],
                    help="PCG tolerance per Newton iteration: fixed 1e-10, or Eisenstat-Walker forcing terms")
    ap.add_argument("--study-eta-max", type=float, default=1e-4, help="largest Eisenstat-Walker tolerance")
    ap.add_argument("--study-save-u", default=None, help="directory for each form's final displacements (.npy)")
    ap.add_argument("--study-lin-maxit", type=int, default=50000)
    ap.add_argument("--study-no-extrapolate", action="store_true",
                    help="start every step from zero instead of the scaled previous increment")
    ap.add_argument("--study-no-adaptive", action="store_true", help="no subdivision of failing steps")
    ap.add_argument("--study-formulation", default="disp", choices=["disp", "bbar", "small_bbar"],
                    help="brick formulation of the precision study: displacement (finite strain), b-bar, or "
                         "small-displacement b-bar")
    ap.add_argument("--type-study", action="store_true",
                    help="time each element type's tangent and recovery alone (hex20, tet10, hex8)")
    ap.add_argument("--batched-study", action="store_true",
                    help="instead of the bench line: Newton solves of the mixed-type bars, FP64 and FP32 tangent")
    ap.add_argument("--study-section", type=int, default=32, help="cells per side of the bars' section")
    ap.add_argument("--crystal-study", action="store_true",
                    help="instead of the bench line: Newton solves of the mm10 polycrystal per tangent form")
    return ap.parse_args()


def build_workload(n, **opts):
    """opts: element formulation (geonl, bbar) -- the default is the
    finite-strain displacement brick."""
    from warp3d_gb300.model import Bilinear, Model, cube_mesh
    coords, incid = cube_mesh(n, jitter=0.1, seed=12345)
    mat = Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0, beta=1.0)
    model = Model(coords, incid, block_size=128, materials=[mat], **opts)
    X = coords
    # load step 1: homogeneous 1% tension with plastic lateral contraction
    F1 = np.diag([1 - 0.005, 1 - 0.005, 1 + 0.01])
    u1 = ((F1 - np.eye(3)) @ X.T).T.ravel()
    # Newton-iteration increment of the next step: 0.1% more, perturbed
    rng = np.random.Generator(np.random.PCG64(2024))
    dF = np.diag([-0.0005, -0.0005, 0.001])
    du = ((dF @ X.T).T + rng.normal(0.0, 2e-5, X.shape)).ravel()
    return model, u1, du


def build_batched_workload(target, seed=2025, ny=64, nz=64):
    """Mixed-type workload: bars of 8-node bricks, 20-node bricks and
    10-node tetrahedra (60/25/15% of `target` elements), random block
    sizes in [16, 128] and per-block yield stresses."""
    from warp3d_gb300 import abi
    from warp3d_gb300.model import Bilinear, Model, Part, mixed_mesh, random_spans
    a = ny * nz
    nx = (max(1, round(0.60 * target / a)), max(1, round(0.25 * target / a)), max(1, round(0.15 * target / (6 * a))))
    coords, parts, origins = mixed_mesh([(abi.ETYPE_L3DISOP, nx[0]), (abi.ETYPE_Q3DISOP, nx[1]),
                                         (abi.ETYPE_TET10, nx[2])], ny, nz, jitter=0.05, seed=seed)
    rng = np.random.Generator(np.random.PCG64(seed))
    plist = []
    for etype, inc in parts:
        spans = random_spans(inc.shape[0], rng, 16, 128)
        mats = [Bilinear.from_hprime(200000.0, 0.3, float(rng.uniform(250.0, 550.0)), 2000.0) for _ in spans]
        plist.append(Part(etype, inc, spans, mats))
    model = Model(coords, parts=plist)
    X = coords
    F1 = np.diag([1 - 0.005, 1 - 0.005, 1 + 0.01])
    u1 = ((F1 - np.eye(3)) @ X.T).T.ravel()
    r2 = np.random.Generator(np.random.PCG64(seed + 1))
    dF = np.diag([-0.0005, -0.0005, 0.001])
    du = ((dF @ X.T).T + r2.normal(0.0, 2e-5, X.shape)).ravel()
    return model, u1, du, nx, origins


def bench_batched(args, dev, local):
    """Batching-form line: autotuned schedule + graph replay, FP64 and FP32
    tangent, next to per-type launches."""
    import torch
    from warp3d_gb300 import abi
    from warp3d_gb300.engine import Engine
    t0 = time.perf_counter()
    model, u1, du, nx, _ = build_batched_workload(args.batched_elems)
    t_build = time.perf_counter() - t0
    ne = model.noelem
    counts = {}
    for t, sp in zip(model.block_etype, model.spans):
        counts[t] = counts.get(t, 0) + sp
    eng = Engine(model, device=local)
    tc = torch.from_numpy(model.c).to(dev)
    tz = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    tu = torch.from_numpy(u1).to(dev)
    tdu = torch.from_numpy(du).to(dev)
    tifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    p = (tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr())
    both = abi.ITER_RECOVER | abi.ITER_TANGENT
    with torch.cuda.stream(stream):   # load step 1 to 1% strain, then the state at n
        eng.recover_dev(1, 1, False, tc.data_ptr(), tz.data_ptr(), tu.data_ptr(), tifv.data_ptr(), sh)
    torch.cuda.synchronize()
    assert eng.recover_info()[0] == 0
    eng.update()

    def time_graph():
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                eng.iteration_dev(2, 1, False, both, *p, sh)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches = 0
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(args.steps):
                eng.iteration_dev(2, 1, False, both, *p, sh)
                launches += eng.last_launch_count()
            e1.record(stream)
        torch.cuda.synchronize()
        assert eng.recover_info()[0] == 0
        return e0.elapsed_time(e1) / args.steps, launches

    def time_direct():
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                eng.recover_dev(2, 1, False, *p, sh)
                eng.tanstf_dev(2, 1, *p[:3], sh)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(args.steps):
                eng.recover_dev(2, 1, False, *p, sh)
                eng.tanstf_dev(2, 1, *p[:3], sh)
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    out = {}
    for name, prec in (("plain_fp64", abi.TANGENT_FP64), ("mixed", abi.TANGENT_FP32)):
        eng.set_precision(prec)
        eng.set_schedule(mode=abi.SCHED_PER_TYPE)
        ms_pt = time_direct()
        t1 = time.perf_counter()
        sched, tuned_ms = eng.autotune(2, 1, False, *p, sh, reps=2)
        t_tune = time.perf_counter() - t1
        # the single persistent launch per kernel against per-type launches,
        # each replayed from its graph (the autotuner's choice is among them
        # or a persistent variant with another occupancy or grain)
        table = {}
        for label, kw in (("per_type", dict(mode=abi.SCHED_PER_TYPE)),
                          ("persistent_heavy_first", dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_HEAVY_FIRST)),
                          ("persistent_block_order", dict(mode=abi.SCHED_PERSISTENT, order=abi.ORDER_BLOCKS))):
            eng.set_schedule(**kw)
            table[label] = round(time_graph()[0], 4)
        eng.set_schedule(**sched)
        ms, launches = time_graph()
        out[name] = {"value": ne / (ms * 1e-3), "ms_per_step": ms, "schedule": sched,
                     "schedules_ms": table,
                     "autotune_best_ms": tuned_ms, "autotune_s": t_tune,
                     "per_type_direct": {"value": ne / (ms_pt * 1e-3), "ms_per_step": ms_pt},
                     "gpu_launches": launches}
    out["mixed"]["speedup_vs_plain"] = out["plain_fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    if not args.no_parity:
        # 16 blocks of each element type against the oracle, same state
        eng.set_schedule(mode=abi.SCHED_PER_TYPE)
        blocks = spread_blocks(model, 16, types=(abi.ETYPE_L3DISOP, abi.ETYPE_Q3DISOP, abi.ETYPE_TET10))
        out["parity"] = parity_sample(eng, model, blocks, 2, 1, False, model.c, u1, du, p, stream,
                                      precisions=(("fp32", abi.TANGENT_FP32), ("tf32", abi.TANGENT_TF32)))
    names = {abi.ETYPE_L3DISOP: "hex8", abi.ETYPE_Q3DISOP: "hex20", abi.ETYPE_TET10: "tet10"}
    res = {"workload": "mixed hex8/hex20/tet10 bars 64x64 cells in section, random blocks [16,128], "
                       "per-block yield U(250,550) MPa, jitter 0.05h, 1 Newton iteration = recovery + tangent",
           "elements": ne, "elements_by_type": {names[k]: v for k, v in counts.items()},
           "bars_nx": {"hex8": nx[0], "hex20": nx[1], "tet10": nx[2]}, "blocks": model.nelblk,
           "gauss_points": int(sum(s * g for s, g in zip(model.spans, model.block_ngp))),
           "model_build_s": t_build, **out}
    eng.close()
    return res


def bench_crystal(args, dev, local, with_cpu):
    """mm10 line: 1% tension in 10 homogeneous steps, then timed iterations."""
    import torch
    from warp3d_gb300 import abi
    from warp3d_gb300.engine import Engine
    from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
    n = args.crystal_n
    coords, incid = cube_mesh(n)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(n ** 3, 4242), dt=1.0)
    ne = model.noelem
    X = coords
    strain = lambda k: ((np.diag([-0.0005 * k, -0.0005 * k, 0.001 * k])) @ X.T).T.ravel()   # k x 0.1%
    eng = Engine(model, device=local)
    tc = torch.from_numpy(model.c).to(dev)
    tifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    # 1% tension in steps of 0.1%; a step whose local solves fail at some
    # Gauss point (status W3G_LOCAL_FAIL) is cut in half and retried, as
    # WARP3D's adaptive step control does with material_cut_step
    t0 = time.perf_counter()
    level, h, step, cuts = 0.0, 1.0, 0, 0
    while level < 10.0 - 1e-9:
        h = min(h, 10.0 - level)
        tu = torch.from_numpy(strain(level)).to(dev)
        tdu = torch.from_numpy(strain(level + h) - strain(level)).to(dev)
        with torch.cuda.stream(stream):
            eng.recover_dev(step + 1, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), sh)
        torch.cuda.synchronize()
        st, _ = eng.recover_info()
        if st != 0:
            h *= 0.5
            cuts += 1
            if h < 1e-3:
                eng.close()
                return {"error": f"load level {level}: status {st} after {cuts} cuts"}
            continue
        eng.update()
        step += 1
        level += h
        h = min(1.0, 2.0 * h)
    t_load = time.perf_counter() - t0
    rng = np.random.Generator(np.random.PCG64(11))
    u = strain(level)
    h_last = 0.25
    du = strain(level + h_last) - strain(level) + rng.normal(0.0, 1e-7, model.nodof)
    tu = torch.from_numpy(u).to(dev)
    tdu = torch.from_numpy(du).to(dev)
    p = (tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr())
    both = abi.ITER_RECOVER | abi.ITER_TANGENT

    def timed(what, steps):
        with torch.cuda.stream(stream):
            for _ in range(max(2, args.warmup)):
                eng.iteration_dev(step + 1, 1, False, what, *p, sh)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches = 0
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                eng.iteration_dev(step + 1, 1, False, what, *p, sh)
                launches += eng.last_launch_count()
            e1.record(stream)
        torch.cuda.synchronize()
        assert eng.recover_info()[0] == 0
        return e0.elapsed_time(e1) / steps, launches

    steps = max(3, args.steps // 2)
    out = {}
    for order in (abi.ORDER_BLOCKS, abi.ORDER_HEAVY_FIRST):
        eng.set_schedule(mode=abi.SCHED_PER_TYPE, order=order)
        ms_rec, _ = timed(abi.ITER_RECOVER, steps)
        out["recovery_ms_" + ("natural_order" if order == abi.ORDER_BLOCKS else "sorted_queue")] = ms_rec
    its = eng.local_iterations()
    for name, prec in (("plain_fp64", abi.TANGENT_FP64), ("mixed", abi.TANGENT_FP32),
                       ("mixed_tf32", abi.TANGENT_TF32)):
        eng.set_precision(prec)
        ms, launches = timed(both, steps)
        out[name] = {"value": ne / (ms * 1e-3), "ms_per_step": ms, "gpu_launches": launches}
    for name in ("mixed", "mixed_tf32"):
        out[name]["speedup_vs_plain"] = out["plain_fp64"]["ms_per_step"] / out[name]["ms_per_step"]
    out["mixed_tf32"]["dtype"] = "tangent TF32 on the tensor cores (tcgen05), recovery fp64"
    eng.set_precision(abi.TANGENT_FP64)
    hist = np.bincount(its, minlength=1)
    out["local_newton_iterations"] = {"min": int(its.min()), "mean": float(its.mean()), "max": int(its.max()),
                                      "p99": float(np.percentile(its, 99)),
                                      "histogram": {int(k): int(v) for k, v in enumerate(hist) if v}}
    if not args.no_parity:
        eng.set_schedule(mode=abi.SCHED_PER_TYPE, order=abi.ORDER_HEAVY_FIRST)
        out["parity"] = parity_sample(eng, model, spread_blocks(model, 16), step + 1, 1, False, model.c, u, du, p,
                                      stream, precisions=(("fp32", abi.TANGENT_FP32), ("tf32", abi.TANGENT_TF32)))
    if with_cpu:
        # CPU baseline leg: the oracle on the first 16 blocks (2,048
        # elements) of the same state
        import oracle
        st = model.new_state()
        eng.download(st)
        nb = min(16, model.nelblk)
        sub = Model(coords, model.incid[:nb * 128], materials=[Crystal()], angles=model.elem_angles[:nb * 128], dt=1.0)
        sst = sub.new_state()
        for name in sst.NAMES:
            setattr(sst, name, [a.copy() for a in getattr(st, name)[:nb]])
        ora = oracle.Oracle(sub, state=sst, threads=host_threads(), fast=True)
        ifv = np.zeros(model.nodof)
        est = sub.estiff_blocks()
        t0 = time.perf_counter()
        reps = 2
        for _ in range(reps):
            ora.recover(step + 1, 1, False, model.c, u, du, ifv)
            ora.tanstf(step + 1, 1, model.c, u, du, est)
        t_cpu = (time.perf_counter() - t0) / reps
        out["cpu_baseline"] = {"value": sub.noelem / t_cpu, "unit": UNIT, "cores": host_threads(), "kind": "port",
                               "sample": f"{sub.noelem} elements ({nb} blocks of 128) of the same state, {reps} iterations",
                               "build": oracle.FAST_FLAGS}
    eng.close()
    return {"workload": f"{n}^3 hex8 l3disop geonl, mm10 fcc Voce (tau_y 90, tau_v 200, theta_0 500 MPa, n 20), "
                        "random orientations, state after 1% tension in 10 steps",
            "elements": ne, "gauss_points": ne * 8, "load_s": t_load, "load_steps": step, "step_cuts": cuts,
            "timed_increment": f"{0.1 * h_last:.3f}% axial strain (+ noise 1e-7)", **out}


# other formulations of the same brick, timed on the 64^3 cube's mesh and
# state: WARP3D's default l3disop (b-bar, finite strain) and the
# small-displacement b-bar brick of its published 18,081-element model
FORMULATIONS = {"bbar": dict(bbar=True), "small_bbar": dict(geonl=False, bbar=True)}


def bench_formulations(args, dev, local):
    import torch
    from warp3d_gb300 import abi
    from warp3d_gb300.engine import Engine
    out = {}
    for name, opts in FORMULATIONS.items():
        model, u1, du = build_workload(args.n, **opts)
        ne = model.noelem
        eng = Engine(model, device=local)
        ifv_h = np.zeros(model.nodof)
        assert eng.recover(1, 1, False, model.c, np.zeros(model.nodof), u1, ifv_h)[0] == 0
        eng.update()
        tc = torch.from_numpy(model.c).to(dev)
        tu = torch.from_numpy(u1).to(dev)
        tdu = torch.from_numpy(du).to(dev)
        tifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
        stream = torch.cuda.Stream(device=dev)
        sh = stream.cuda_stream
        res = {"workload": f"{args.n}^3 hex8 l3disop {'geonl' if opts.get('geonl', True) else 'small displacement'}"
                           f" b-bar, mm01, state and increment as the headline"}
        for pname, prec in (("fp64", abi.TANGENT_FP64), ("fp32", abi.TANGENT_FP32), ("tf32", abi.TANGENT_TF32)):
            eng.set_precision(prec)
            with torch.cuda.stream(stream):
                for _ in range(args.warmup):
                    eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), sh)
                    eng.recover_dev(2, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), sh)
            torch.cuda.synchronize()
            evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps + 1)]
            with torch.cuda.stream(stream):
                evs[0].record(stream)
                for k in range(args.steps):
                    eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), sh)
                    evs[2 * k + 1].record(stream)
                    eng.recover_dev(2, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), sh)
                    evs[2 * k + 2].record(stream)
            torch.cuda.synchronize()
            assert eng.recover_info()[0] == 0
            t_tan = sum(evs[2 * k].elapsed_time(evs[2 * k + 1]) for k in range(args.steps)) / args.steps
            t_rec = sum(evs[2 * k + 1].elapsed_time(evs[2 * k + 2]) for k in range(args.steps)) / args.steps
            ms = evs[0].elapsed_time(evs[-1]) / args.steps
            res[pname] = {"value": ne / (ms * 1e-3), "ms_per_step": ms, "tangent_ms": t_tan, "recovery_ms": t_rec}
        res["mixed_speedup"] = res["fp64"]["ms_per_step"] / res["fp32"]["ms_per_step"]
        if name == "small_bbar":
            # the only figures WARP3D publishes for this path: its 18,081-element
            # small-displacement b-bar example (mm01 with temperature curves), 10
            # OpenMP threads on an Intel Mac (example_3_nonlinear/output_20C_temp)
            res["reference_published"] = {"value": 0.68e6, "tangent_elem_s": 1.54e6, "recovery_elem_s": 1.22e6,
                                          "unit": UNIT, "hardware": "Intel Mac, 10 OpenMP threads (ifort + MKL)"}
        out[name] = res
        eng.close()
        del tc, tu, tdu, tifv
        torch.cuda.empty_cache()
    return out


def type_study(args, dev):
    """One Newton iteration's element work per element type alone, FP64 and
    with the FP32 tangent (and for bricks the tensor-core tangents): 40^3 20-node bricks, 40^3 x 6 10-node
    tetrahedra, n^3 8-node bricks (jitter 0.05h, mm01, blocks of 128;
    state after one step to 1% tension; CUDA events over 5 calls each)."""
    import torch
    from warp3d_gb300 import abi
    from warp3d_gb300.engine import Engine
    from warp3d_gb300.model import Bilinear, Model, cube_mesh, cube_mesh_hex20, cube_mesh_tet10
    out = {}
    for name, mesh, n, et in (("hex20", cube_mesh_hex20, 40, abi.ETYPE_Q3DISOP),
                              ("tet10", cube_mesh_tet10, 40, abi.ETYPE_TET10),
                              ("hex8", cube_mesh, args.n, abi.ETYPE_L3DISOP)):
        coords, incid = mesh(n, jitter=0.05, seed=3)
        model = Model(coords, incid, etype=et, materials=[Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)])
        eng = Engine(model)
        u1 = (np.diag([-0.005, -0.005, 0.01]) @ coords.T).T.ravel()
        assert eng.recover(1, 1, False, model.c, np.zeros(model.nodof), u1, np.zeros(model.nodof))[0] == 0
        eng.update()
        du = (np.diag([-0.0005, -0.0005, 0.001]) @ coords.T).T.ravel()
        tc, tu, tdu = (torch.from_numpy(a).to(dev) for a in (model.c, u1, du))
        tifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
        res = {"elements": model.noelem}
        forms = [("fp64", abi.TANGENT_FP64), ("fp32", abi.TANGENT_FP32)]
        if et != abi.ETYPE_TET10:   # bricks: the tensor-core forms too
            forms += [("tf32", abi.TANGENT_TF32), ("bf16", abi.TANGENT_BF16), ("tf32x3", abi.TANGENT_TF32X3),
                      ("bf16x3", abi.TANGENT_BF16X3)]
        for pname, prec in forms:
            eng.set_precision(prec)
            for _ in range(max(3, args.warmup)):
                eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), 0)
                eng.recover_dev(2, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), 0)
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record()
            for _ in range(5):
                eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), 0)
            ev[1].record()
            for _ in range(5):
                eng.recover_dev(2, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), 0)
            ev[2].record()
            torch.cuda.synchronize()
            res[pname] = {"tangent_ms": ev[0].elapsed_time(ev[1]) / 5, "recover_ms": ev[1].elapsed_time(ev[2]) / 5}
        out[name] = res
        eng.close()
        del tc, tu, tdu, tifv
        torch.cuda.empty_cache()
    return out


def sample_clocks():
    try:
        return subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
             "--format=csv,noheader,nounits", "-lms", "200"],
            stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except OSError:
        return None


def finish_clocks(proc, device_index):
    if proc is None:
        return None
    proc.terminate()
    try:
        out, _ = proc.communicate(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
        out, _ = proc.communicate()
    mhz, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.strip().splitlines():
        f = [x.strip() for x in line.split(",")]
        if len(f) < 9 or f[0] != str(device_index):
            continue
        try:
            mhz.append(float(f[1]))
            mx = float(f[2])
        except ValueError:
            continue
        for nm, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(nm)
    if not mhz:
        return None
    return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(mhz)}


def load_traffic():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


# ---- parity at the benchmark's own sizes ---------------------------------
# The oracle (the CPU restatement, checker build) replays one Newton
# iteration of element work on a sample of blocks of the benchmark model:
# the sample blocks' state is read from the device before a GPU iteration,
# the GPU iteration runs on the whole model, its outputs for the sample
# blocks are read back, and the oracle runs the same iteration on a model
# made of the sample blocks alone (same nodes, materials, orientations),
# from the same state. Outside every timed region.

PARITY_ARRAYS = ("urcs_n1", "eps_n1", "rot_n1", "history1", "cep", "einfvec", "element_vol")


def sub_model(model, blocks):
    """A model holding only `blocks` of `model` (one part per block, in the
    given order) over the nodes they use, and that node map."""
    from warp3d_gb300.model import Model, Part
    incs = [model._block_incid[b] for b in blocks]
    used = np.unique(np.concatenate([i.ravel() for i in incs]))
    remap = -np.ones(model.nnode, dtype=np.int64)
    remap[used] = np.arange(len(used))
    parts = [Part(model.block_etype[b], remap[model._block_incid[b]], [model.spans[b]], [model.block_material[b]])
             for b in blocks]
    angles = None
    if model.crystals:
        angles = np.concatenate([model.elem_angles[model.felem[b]:model.felem[b] + model.spans[b]] for b in blocks])
    sub = Model(model.coords[used], parts=parts, geonl=model.geonl, bbar=model.bbar, qbar=model.qbar,
                angles=angles, dt=model.dt, eps_bbar=model.eps_bbar, asymmetric=model.asymmetric)
    dofs = (3 * used[:, None] + np.arange(3)[None, :]).ravel()
    return sub, dofs


def _scatter_struct(model, sub_state, blocks, names):
    """BlockState of the full model whose block pointers point into
    sub_state for `blocks` and are NULL elsewhere."""
    from warp3d_gb300 import abi
    st, keep = abi.BlockState(), []
    for name in names:
        addr = np.zeros(model.nelblk, dtype=np.uintp)
        for k, b in enumerate(blocks):
            addr[b] = getattr(sub_state, name)[k].__array_interface__["data"][0]
        arr = (C.c_void_p * model.nelblk).from_buffer(addr)
        keep.append((addr, arr))
        setattr(st, name, C.cast(arr, C.POINTER(C.POINTER(C.c_double))))
    return st, keep


def _download_blocks(eng, model, sub, blocks, names):
    from warp3d_gb300 import abi
    state = sub.new_state()
    st, keep = _scatter_struct(model, state, blocks, names)
    abi.check(eng.lib, eng.lib.w3g_state_download(eng.ctx, C.byref(st)))
    del keep
    return state


def _estiff_blocks(eng, model, blocks):
    """Element stiffnesses of `blocks` from the device (FP64 or FP32, as the
    engine's current precision form stores them), as float64 (span, rows)."""
    import torch
    from warp3d_gb300 import abi
    torch.cuda.synchronize()
    ptr, _ = eng.estiff_device()
    f32 = eng.precision != abi.TANGENT_FP64
    sizes = np.array(model.spans, dtype=np.int64) * np.array(model.block_ek_rows, dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    cudart = C.CDLL("libcudart.so")
    out = []
    for b in blocks:
        a = np.empty((model.spans[b], model.block_ek_rows[b]), dtype=np.float32 if f32 else np.float64)
        rc = cudart.cudaMemcpy(C.c_void_p(a.ctypes.data), C.c_void_p(ptr + int(offs[b]) * a.itemsize),
                               C.c_size_t(a.nbytes), 2)
        assert rc == 0, f"cudaMemcpy {rc}"
        out.append(a.astype(np.float64))
    return out


def _ke_err(got, ref):
    """max over elements of max|dKe| / max|Ke| (per-element relative)."""
    worst = 0.0
    for g, o in zip(got, ref):
        den = np.max(np.abs(o), axis=1)
        worst = max(worst, float(np.max(np.max(np.abs(g - o), axis=1) / np.where(den > 0, den, 1.0))))
    return worst


def parity_sample(eng, model, blocks, step, it, extrap, c, u, du, dptrs, stream, precisions=()):
    """One GPU Newton iteration (recovery, then tangent) of the whole model
    against the oracle on `blocks`; returns the max relative error per
    output array, per-element for Ke, and for each precision form in
    `precisions` ((name, code) pairs) its Ke error against the oracle's
    FP64 Ke on the same blocks."""
    import torch
    import oracle
    from warp3d_gb300 import abi
    from warp3d_gb300.model import HostState
    blocks = [int(b) for b in blocks]
    sub, dofs = sub_model(model, blocks)
    prec0 = eng.precision
    eng.set_precision(abi.TANGENT_FP64)
    pre = _download_blocks(eng, model, sub, blocks, HostState.NAMES)
    d_c, d_u, d_du, d_ifv = dptrs
    with torch.cuda.stream(stream):
        eng.recover_dev(step, it, extrap, d_c, d_u, d_du, d_ifv, stream.cuda_stream)
        eng.tanstf_dev(step, it, d_c, d_u, d_du, stream.cuda_stream)
    torch.cuda.synchronize()
    st_gpu, _ = eng.recover_info()
    post = _download_blocks(eng, model, sub, blocks, PARITY_ARRAYS)
    ke_gpu = _estiff_blocks(eng, model, blocks)
    ora = oracle.Oracle(sub, state=pre, threads=host_threads())
    ifv = np.zeros(sub.nodof)
    st_ora, _ = ora.recover(step, it, extrap, sub.c, np.ascontiguousarray(u[dofs]), np.ascontiguousarray(du[dofs]),
                            ifv)
    ke_ora = sub.estiff_blocks()
    ora.tanstf(step, it, sub.c, np.ascontiguousarray(u[dofs]), np.ascontiguousarray(du[dofs]), ke_ora)
    res = {"blocks": len(blocks), "elements": sub.noelem, "status_gpu": int(st_gpu), "status_oracle": int(st_ora)}
    for name in PARITY_ARRAYS:
        g = np.concatenate([a.ravel() for a in getattr(post, name)])
        o = np.concatenate([a.ravel() for a in getattr(ora.state, name)])
        den = float(np.max(np.abs(o)))
        res[name] = float(np.max(np.abs(g - o)) / den) if den > 0 else float(np.max(np.abs(g)))
    res["estiff"] = _ke_err(ke_gpu, ke_ora)
    res["max_fp64"] = max(res[k] for k in (*PARITY_ARRAYS, "estiff"))
    if precisions:
        res["estiff_precision_forms"] = {}
        for name, code in precisions:
            eng.set_precision(code)
            with torch.cuda.stream(stream):
                eng.tanstf_dev(step, it, d_c, d_u, d_du, stream.cuda_stream)
            torch.cuda.synchronize()
            res["estiff_precision_forms"][name] = _ke_err(_estiff_blocks(eng, model, blocks), ke_ora)
    eng.set_precision(prec0)
    return res


def spread_blocks(model, k, types=None):
    """k blocks spread evenly over the model (per element type if `types`)."""
    if types is None:
        return np.unique(np.linspace(0, model.nelblk - 1, k).round().astype(int)).tolist()
    out = []
    for t in types:
        bs = [b for b in range(model.nelblk) if model.block_etype[b] == t]
        if bs:
            out += [bs[i] for i in np.unique(np.linspace(0, len(bs) - 1, k).round().astype(int))]
    return out


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline(model_n, nblocks, threads, reps=8, warmup=1):
    """Times the oracle (CPU restatement, OpenMP over blocks, compiled with
    multiply-add contraction as WARP3D's ifort -O3 build is) on the first
    `nblocks` element blocks of the same workload (None: all of it): one
    recovery + one tangent per rep, like a Newton iteration."""
    import oracle
    from warp3d_gb300.model import Bilinear, Model, cube_mesh
    coords, incid = cube_mesh(model_n, jitter=0.1, seed=12345)
    ne = incid.shape[0] if nblocks is None else min(nblocks * 128, incid.shape[0])
    used = np.unique(incid[:ne])
    remap = -np.ones(coords.shape[0], dtype=np.int64)
    remap[used] = np.arange(len(used))
    sub = Model(coords[used], remap[incid[:ne]], block_size=128,
                materials=[Bilinear.from_hprime(200000.0, 0.3, 400.0, 2000.0)])
    X = sub.coords
    F1 = np.diag([1 - 0.005, 1 - 0.005, 1 + 0.01])
    u1 = ((F1 - np.eye(3)) @ X.T).T.ravel()
    rng = np.random.Generator(np.random.PCG64(2024))
    du = ((np.diag([-0.0005, -0.0005, 0.001]) @ X.T).T + rng.normal(0.0, 2e-5, X.shape)).ravel()
    ora = oracle.Oracle(sub, threads=threads, deterministic=False, fast=True)
    ifv = np.zeros(sub.nodof)
    ora.recover(1, 1, False, sub.c, np.zeros(sub.nodof), u1, ifv)
    ora.update()
    est = [np.zeros((s, sub.utsz)) for s in sub.spans]
    for _ in range(max(1, warmup)):
        ora.recover(2, 1, False, sub.c, u1, du, ifv)
        ora.tanstf(2, 1, sub.c, u1, du, est)
    t_rec = t_tan = 0.0
    for _ in range(reps):
        t0 = time.perf_counter()
        ora.recover(2, 1, False, sub.c, u1, du, ifv)
        t1 = time.perf_counter()
        ora.tanstf(2, 1, sub.c, u1, du, est)
        t2 = time.perf_counter()
        t_rec += t1 - t0
        t_tan += t2 - t1
    t_rec /= reps
    t_tan /= reps
    what = "all" if nblocks is None or ne == incid.shape[0] else "the first"
    return {"value": ne / (t_rec + t_tan), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} {ne} elements ({len(sub.spans)} blocks of 128) of the {model_n}^3 workload, "
                      f"{reps} iterations after {max(1, warmup)} warm-up",
            "cpu": cpu_model(), "build": oracle.FAST_FLAGS,
            "tangent_elem_per_s": ne / t_tan, "recovery_elem_per_s": ne / t_rec}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def whole_job_throughput(units_per_rank, ms_local, world, dist=None, device="cpu"):
    """Replicas (one independent copy of the workload per rank, no data-path
    collective): the step time is the maximum over ranks and the value is
    all ranks' units over it. Returns (units/s, max ms)."""
    t_step = ms_local
    if dist is not None:
        import torch
        t = torch.tensor([ms_local], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step = float(t.item())
    return world * units_per_rank / (t_step * 1e-3), t_step


def reference_arm(args, rank, world):
    """The reference's CPU path on the host cores: the oracle's contracted
    build on the whole headline workload (all 262,144 elements at 64^3),
    the same warm-up and timed step counts as the GPU arm."""
    if rank != 0:
        return
    threads = host_threads()
    cb = cpu_baseline(args.n, None, threads, reps=args.steps, warmup=args.warmup)
    ne = args.n ** 3
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * ne / cb["value"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.n}^3 hex8 l3disop geonl (jitter 0.1h), mm01 bilinear, blocks of 128, "
                               f"1 Newton iteration = tangent + recovery",
                   "elements": ne, "gauss_points": ne * 8, "sample": cb["sample"]},
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "cpu", "build")},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "WARP3D itself (Fortran + Intel MKL) cannot be built here; the reference arm times the "
                "oracle, a C++ restatement of the same routines compiled with multiply-add contraction, "
                "OpenMP over blocks on all host threads",
    }
    print(json.dumps(line), flush=True)


def hbm_peak_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f).get("hbm_gbs")
    except OSError:
        return None


def bench_solver(args, eng, model, tc, tu, tdu, dev):
    """Device assembly of K from the resident FP64 element stiffnesses and
    the Jacobi-PCG iteration on the same workload; both HBM-bound. Bytes:
    assembly = contributions x (4 B index + 8 B value) + coefficients x
    (4 B pointer + 8 B write); one CG iteration = nnz x (8 B value + 4/3 B
    column: a node's three rows share their column indices) + nodof x
    109 B (row pointers, mask, the gathered direction, and the vector
    updates' reads and writes)."""
    import torch
    from warp3d_gb300.newton import uniaxial_bcs
    from warp3d_gb300.solver import DeviceCsr
    n = args.n
    eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr())
    t0 = time.perf_counter()
    csr = DeviceCsr(eng)
    setup_s = time.perf_counter() - t0
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for _ in range(2):
        csr.assemble()
    torch.cuda.synchronize()
    reps = 5
    ev[0].record()
    for _ in range(reps):
        csr.assemble()
    ev[1].record()
    torch.cuda.synchronize()
    asm_ms = ev[0].elapsed_time(ev[1]) / reps
    ncontrib = int(sum(model.block_totdof[b] ** 2 * model.spans[b] for b in range(model.nelblk)))
    asm_bytes = 12 * ncontrib + 12 * csr.nnz
    fixed, _ = uniaxial_bcs(model, (n, n, n))
    mask = torch.zeros(model.nodof, dtype=torch.uint8, device=dev)
    mask[torch.from_numpy(fixed).to(dev)] = 1
    g = torch.Generator(device="cpu").manual_seed(11)
    b = torch.randn(model.nodof, generator=g, dtype=torch.float64).to(dev)
    x = torch.zeros_like(b)
    csr.pcg(mask.data_ptr(), b.data_ptr(), 1.0, x.data_ptr(), 0.0, 32)   # warm-up, graph capture
    its_req = 320
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st, its, rel = csr.pcg(mask.data_ptr(), b.data_ptr(), 1.0, x.data_ptr(), 0.0, its_req)
    torch.cuda.synchronize()
    it_ms = 1e3 * (time.perf_counter() - t0) / max(its, 1)
    # iterations to converge on the same right-hand side
    st_c, its_c, rel_c = csr.pcg(mask.data_ptr(), b.data_ptr(), 1.0, x.data_ptr(), 1e-10, 50000)
    it_bytes = (8 + 4 / 3) * csr.nnz + 109 * model.nodof
    peak = hbm_peak_gbs()
    out = {"dofs": model.nodof, "nnz": csr.nnz, "contributions": ncontrib, "pattern_setup_s": setup_s,
           "assemble_ms": asm_ms, "assemble_gbs": asm_bytes / (asm_ms * 1e-3) / 1e9,
           "pcg_iterations_timed": its, "pcg_iteration_ms": it_ms, "pcg_iterations_to_1e-10": its_c,
           "pcg_iteration_gbs": it_bytes / (it_ms * 1e-3) / 1e9, "hbm_peak_gbs": peak}
    if peak:
        out["assemble_frac"] = out["assemble_gbs"] / peak
        out["pcg_iteration_frac"] = out["pcg_iteration_gbs"] / peak
    csr.close()
    return out


STUDY_FORMS = {"fp64": 0, "fp32": 1, "tf32": 2, "bf16": 3, "tf32x3": 4, "bf16x3": 5}   # abi.TANGENT_*


def newton_forms(args, model, fixed, topz, nz, names, eng, csr):
    """Runs the displacement-controlled load history on the device once per
    tangent form (DeviceNewtonDriver: extrapolated starts, adaptive
    subdivision with step 1 included); returns per-form records, the FP64
    run's displacements and its converged end state."""
    import torch
    from warp3d_gb300.solver import DeviceNewtonDriver
    initial = model.new_state()
    eng.set_precision(STUDY_FORMS["fp64"])
    eng.download(initial)
    forms, u_ref, end_state, steps_ref = {}, None, None, 0
    for name in names:
        eng.set_precision(STUDY_FORMS[name])
        eng.upload(initial)
        drv = DeviceNewtonDriver(model, eng, fixed, tol=1e-8, maxit=args.study_maxit, lin_rtol=1e-10,
                                 lin_maxit=args.study_lin_maxit, csr=csr, extrapolate=not args.study_no_extrapolate,
                                 adaptive=not args.study_no_adaptive, adaptive_step1=True,
                                 forcing=args.study_forcing, eta_max=args.study_eta_max)
        rec = {"steps": [], "failed": None}
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for st in range(1, args.study_steps + 1):
            imp = np.zeros(model.nodof)
            imp[topz] = args.study_strain * nz / args.study_steps
            k0, cuts0 = len(drv.history), drv.cuts
            try:
                drv.step(st, imp)
            except RuntimeError as exc:
                rec["failed"] = {"step": st, "reason": str(exc)[:300],
                                 "trace": [[a, b, float(f"{c:.3e}"), None if d is None else float(f"{d:.3e}")]
                                           for a, b, c, d in drv.trace]}
                break
            incs = drv.history[k0:]
            rec["steps"].append({"step": st, "newton": sum(h[1] for h in incs), "increments": len(incs),
                                 "cuts": drv.cuts - cuts0,
                                 "residuals": [[float(f"{r:.3e}") for r in h[2]] for h in incs],
                                 "pcg": [x for _, l in drv.lin_history[k0:] for x in l]})
        torch.cuda.synchronize()
        rec["wall_s"] = time.perf_counter() - t1
        its = [x["newton"] for x in rec["steps"]]
        rec["newton_per_step"] = its
        rec["increments_per_step"] = [x["increments"] for x in rec["steps"]]
        rec["mean_newton_per_step"] = float(np.mean(its)) if its else None
        rec["pcg_total"] = int(sum(sum(x["pcg"]) for x in rec["steps"]))
        u = drv.u
        if args.study_save_u:
            os.makedirs(args.study_save_u, exist_ok=True)
            np.save(os.path.join(args.study_save_u, f"u_{name}.npy"), u)
        if name == "fp64":
            u_ref, steps_ref = u, len(rec["steps"])
            end_state = model.new_state()
            eng.download(end_state)
        elif u_ref is not None and len(rec["steps"]) == steps_ref:
            # the same number of converged steps as the FP64 run (all, or
            # up to the step where both stopped)
            rec["u_rel_err_vs_fp64"] = float(np.max(np.abs(u - u_ref)) / np.max(np.abs(u_ref)))
        forms[name] = rec
        print(f"[study] {name}: newton {its} failed={rec['failed'] is not None} {rec['wall_s']:.1f}s",
              file=sys.stderr, flush=True)
    return forms, u_ref, end_state


def batched_study(args, dev):
    """The batching form's Newton solve: the mixed hex8/hex20/tet10 bars
    (random blocks, per-block yield) in uniaxial tension, plain FP64
    against the FP32 precision form, every iteration on the device."""
    from warp3d_gb300.engine import Engine
    from warp3d_gb300.newton import uniaxial_bcs
    from warp3d_gb300.solver import DeviceCsr
    ny = nz = args.study_section
    model, _, _, nx, origins = build_batched_workload(args.batched_elems, ny=ny, nz=nz)
    fixed, topz = uniaxial_bcs(model, (nx[0], ny, nz), origins=origins)
    t0 = time.perf_counter()
    eng = Engine(model)
    csr = DeviceCsr(eng)
    setup_s = time.perf_counter() - t0
    names = args.study_forms.split(",")
    forms, _, _ = newton_forms(args, model, fixed, topz, nz, names, eng, csr)
    csr.close()
    return {"workload": f"mixed bars hex8/hex20/tet10 ({ny}x{nz} cells in section, nx {list(nx)}), random blocks "
                        f"[16,128], per-block yield U(250,550) MPa; uniaxial {100 * args.study_strain:g}% in "
                        f"{args.study_steps} steps",
            "elements": model.noelem, "blocks": model.nelblk, "dofs": model.nodof, "csr_nnz": csr.nnz,
            "setup_s": setup_s, "newton_tol": 1e-8,
            "pcg_rtol": 1e-10 if args.study_forcing == "fixed" else
            f"Eisenstat-Walker (gamma 0.9, eta_max {args.study_eta_max:g}, floor 1e-10)",
            "forms": forms}


def crystal_study(args, dev):
    """The precision forms on the mm10 polycrystal of the crystal line
    (crystal_n^3 8-node bricks, fcc, Euler angles uniform on SO(3), Voce)
    under uniaxial tension, args.study_strain in args.study_steps equal
    steps, every Newton iteration on the device (element path with the mm10
    local solves, CSR assembly, Jacobi PCG, residual norms) to the 1e-8
    relative residual; a step whose local solves fail is subdivided.
    Per form: Newton iterations per step, PCG iterations, wall time and the
    final displacements' error against the FP64 run."""
    from warp3d_gb300.engine import Engine
    from warp3d_gb300.model import Crystal, Model, cube_mesh, random_orientations
    from warp3d_gb300.newton import uniaxial_bcs
    from warp3d_gb300.solver import DeviceCsr
    n = args.crystal_n
    coords, incid = cube_mesh(n)
    model = Model(coords, incid, materials=[Crystal()], angles=random_orientations(n ** 3, 4242), dt=1.0)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    t0 = time.perf_counter()
    eng = Engine(model)
    csr = DeviceCsr(eng)
    setup_s = time.perf_counter() - t0
    forms, _, _ = newton_forms(args, model, fixed, topz, n, args.study_forms.split(","), eng, csr)
    out = {"workload": f"{n}^3 hex8 mm10 fcc polycrystal (random orientations, Voce), uniaxial "
                       f"{100 * args.study_strain:g}% in {args.study_steps} steps",
           "elements": model.noelem, "dofs": model.nodof, "csr_nnz": csr.nnz, "setup_s": setup_s,
           "newton_tol": 1e-8,
           "pcg_rtol": 1e-10 if args.study_forcing == "fixed" else
           f"Eisenstat-Walker (gamma 0.9, eta_max {args.study_eta_max:g}, floor 1e-10)",
           "forms": forms}
    csr.close()
    eng.close()
    return out


def precision_study(args, dev):
    """The precision forms on the n^3 cube (mm01, jitter 0.1h, blocks of
    128) under uniaxial tension, args.study_strain in args.study_steps
    equal steps, every Newton iteration on the device (element path, CSR
    assembly, Jacobi PCG to 1e-10, residual norms) to the 1e-8 relative
    residual; steps start from the scaled previous increment and a failing
    step is subdivided (4 sub-increments, down to 1/16 of the step, step 1
    included). Per form: Newton iterations per step, PCG iterations, wall
    time, the final displacements' error against the FP64 run; per-element
    Ke error against the FP64 tangent (checked against the oracle by the
    tests) at the converged end state of the FP64 run."""
    import torch
    from warp3d_gb300 import abi
    from warp3d_gb300.engine import Engine
    from warp3d_gb300.newton import uniaxial_bcs
    from warp3d_gb300.solver import DeviceCsr
    forms = {k: v for k, v in STUDY_FORMS.items()}
    n = args.n
    opts = FORMULATIONS.get(args.study_formulation, {})
    model, _, _ = build_workload(n, **opts)
    fixed, topz = uniaxial_bcs(model, (n, n, n))
    t0 = time.perf_counter()
    eng = Engine(model)
    csr = DeviceCsr(eng)
    setup_s = time.perf_counter() - t0
    form = {"disp": "geonl", "bbar": "geonl b-bar", "small_bbar": "small-displacement b-bar"}[args.study_formulation]
    out = {"workload": f"{n}^3 hex8 l3disop {form} (jitter 0.1h), mm01 bilinear, blocks of 128; uniaxial "
                       f"{100 * args.study_strain:g}% in {args.study_steps} steps",
           "elements": model.noelem, "dofs": model.nodof, "csr_nnz": csr.nnz, "setup_s": setup_s,
           "newton_tol": 1e-8, "pcg_rtol": 1e-10, "forms": {}}
    out["forms"], u_ref, end_state = newton_forms(args, model, fixed, topz, n, args.study_forms.split(","), eng, csr)
    # per-element Ke error at the FP64 run's converged end state
    if u_ref is not None:
        tu = torch.from_numpy(u_ref).to(dev)
        tz = torch.zeros_like(tu)
        tc = torch.from_numpy(model.c).to(dev)
        ne, ut = model.noelem, model.utsz

        def ke(prec):
            eng.set_precision(prec)
            eng.upload(end_state)
            eng.tanstf_dev(args.study_steps, 1, tc.data_ptr(), tu.data_ptr(), tz.data_ptr())
            torch.cuda.synchronize()
            p, cnt = eng.estiff_device()
            dt = torch.float64 if prec == abi.TANGENT_FP64 else torch.float32
            t = torch.empty(cnt, dtype=dt, device=dev)
            cudart = C.CDLL("libcudart.so")
            assert cudart.cudaMemcpy(C.c_void_p(t.data_ptr()), C.c_void_p(p), C.c_size_t(t.element_size() * cnt),
                                     3) == 0
            return t.double().reshape(ne, ut)

        k64 = ke(abi.TANGENT_FP64)
        scale = k64.abs().amax(dim=1)
        for name in args.study_forms.split(","):
            if name == "fp64":
                continue
            e = (ke(forms[name]) - k64).abs().amax(dim=1) / scale
            out["forms"][name]["ke_rel_err"] = {"max": float(e.max()), "median": float(e.median()),
                                                "p99": float(torch.quantile(e[:: max(1, ne // 100000)], 0.99))}
        eng.set_precision(abi.TANGENT_FP64)
    csr.close()
    return out


def _r(x, nd=4):
    return None if x is None else float(f"{x:.{nd}g}")


def summarize_mixed(mixed):
    """Headline view of the precision forms: per form the tangent time and
    the iteration's speed-up over plain FP64."""
    if not mixed:
        return None
    out = {"value": _r(mixed["value"]), "speedup_vs_fp64": _r(mixed["speedup_vs_fp64"]),
           "form": mixed.get("form", "fp32"), "dtype": mixed.get("dtype")}
    forms = {"fp32": {"tangent_ms": _r(mixed["fp32"]["tangent_ms"]), "speedup": _r(mixed["fp32"]["speedup_vs_fp64"])}}
    for k, v in (mixed.get("tensor_core") or {}).items():
        forms[k] = {"tangent_ms": _r(v["tangent_ms"]), "speedup": _r(v["speedup_vs_fp64"]),
                    "tangent_hbm_frac": _r(v.get("tangent_hbm_frac"))}
    out["forms"] = forms
    return out


def compact_roofline(rf):
    keep = ("bound", "kernel", "achieved", "peak", "unit", "frac", "traffic", "peak_source")
    out = {k: rf[k] for k in keep if k in rf}
    for k in ("tangent_tc", "recovery"):
        if k in rf:
            out[k] = rf[k]
    return out


def regression_pins():
    """WARP3D's own regression problems replayed through the GPU engine
    (the host-array C-ABI, FP64): verification/test24 (mm01, finite-strain
    b-bar bricks) and verification/test82/voche_model (mm10, bcc, Voce),
    from the committed fixtures; per deck the stress its checker compares,
    WARP3D's value and the relative difference (the checker accepts 1e-4)."""
    out = {}
    try:
        from tests import warp3d_test24 as t24
        from tests import warp3d_test82 as t82
        from warp3d_gb300.engine import Engine
        for name, mod in (("test24_sphere_mm01", t24), ("test82_voce_mm10", t82)):
            d = mod.load()
            t0 = time.perf_counter()
            sig, _, its = mod.solve(Engine, d)
            expected = float(d["expected_answer"])
            out[name] = {"computed": float(sig[0]), "warp3d": expected, "rel": abs(float(sig[0]) / expected - 1.0),
                         "checker_rtol": mod.CHECKER_RTOL, "newton_iterations": int(sum(its)),
                         "s": time.perf_counter() - t0}
    except Exception as exc:   # reported, never fatal to the bench line
        out["error"] = f"{type(exc).__name__}: {str(exc)[:200]}"
    return out


def summarize_parity(p1, batched, crystal, pins=None):
    """Max relative error of every FP64 output array against the oracle,
    per workload, and the precision forms' Ke error."""
    def one(p):
        if not p:
            return None
        d = {"elements": p["elements"], "max_fp64": _r(p["max_fp64"], 3),
             "worst_array": max(PARITY_ARRAYS + ("estiff",), key=lambda k: p[k])}
        if "estiff_precision_forms" in p:
            d["ke_precision_forms"] = {k: _r(v, 3) for k, v in p["estiff_precision_forms"].items()}
        return d
    out = {"hex8_64cube": one(p1), "mixed_1m_batched": one((batched or {}).get("parity")),
           "mm10_32cube": one((crystal or {}).get("parity")), "tolerance_fp64": 1e-12}
    if pins:
        out["warp3d_regression_rel"] = {k: (_r(v["rel"], 3) if isinstance(v, dict) else v) for k, v in pins.items()}
    return out


def summarize_leg(leg):
    if not leg or "plain_fp64" not in leg:
        return leg and {"error": leg.get("error")}
    out = {"elements": leg.get("elements"), "plain_fp64": _r(leg["plain_fp64"]["value"]),
           "plain_ms": _r(leg["plain_fp64"]["ms_per_step"])}
    for k in ("mixed", "mixed_tf32", "mixed_tc"):
        if k in leg:
            out[k] = _r(leg[k]["value"])
            out[k + "_speedup"] = _r(leg[k].get("speedup_vs_plain"))
    if "cpu_baseline" in leg:
        out["cpu_baseline"] = _r(leg["cpu_baseline"]["value"])
    # the batching form: the single persistent launch against per-type
    # launches (graph replays, ms per iteration) and the autotuner's pick
    for k in ("plain_fp64", "mixed"):
        if isinstance(leg.get(k), dict) and "schedules_ms" in leg[k]:
            out[k + "_schedules_ms"] = leg[k]["schedules_ms"]
            out[k + "_tuned_mode"] = leg[k].get("schedule", {}).get("mode")
    return out


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    if args.precision_study:
        print(json.dumps({"precision_study": precision_study(args, dev)}))
        return
    if args.batched_study:
        print(json.dumps({"batched_study": batched_study(args, dev)}))
        return
    if args.type_study:
        print(json.dumps({"type_study": type_study(args, dev)}))
        return
    if args.crystal_study:
        print(json.dumps({"crystal_study": crystal_study(args, dev)}))
        return

    from warp3d_gb300 import abi
    from warp3d_gb300.engine import Engine

    model, u1, du = build_workload(args.n)
    ne = model.noelem
    eng = Engine(model, device=local)
    ifv_h = np.zeros(model.nodof)
    st, _ = eng.recover(1, 1, False, model.c, np.zeros(model.nodof), u1, ifv_h)
    assert st == 0
    eng.update()

    tc = torch.from_numpy(model.c).to(dev)
    tu = torch.from_numpy(u1).to(dev)
    tdu = torch.from_numpy(du).to(dev)
    tifv = torch.zeros(model.nodof, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(precision):
        eng.set_precision(precision)
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), sh)
                eng.recover_dev(2, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), sh)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps + 1)]
        launches = 0
        with torch.cuda.stream(stream):
            evs[0].record(stream)
            for k in range(args.steps):
                eng.tanstf_dev(2, 1, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), sh)
                launches += eng.last_launch_count()
                evs[2 * k + 1].record(stream)
                eng.recover_dev(2, 1, False, tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr(), sh)
                launches += eng.last_launch_count()
                evs[2 * k + 2].record(stream)
        torch.cuda.synchronize()
        barrier()
        t_tan = sum(evs[2 * k].elapsed_time(evs[2 * k + 1]) for k in range(args.steps)) / args.steps
        t_rec = sum(evs[2 * k + 1].elapsed_time(evs[2 * k + 2]) for k in range(args.steps)) / args.steps
        total = evs[0].elapsed_time(evs[-1])
        st, info = eng.recover_info()
        assert st == 0
        return total / args.steps, t_tan, t_rec, launches

    peak = C.c_double()
    abi.check(eng.lib, eng.lib.w3g_measure_fp64_peak(local, C.byref(peak)))
    fp64_peak_tflops = peak.value

    clk = sample_clocks()
    ms64, tan64, rec64, launches64 = timed(abi.TANGENT_FP64)
    clocks = finish_clocks(clk, local)
    mixed = None
    hbm = hbm_peak_gbs()
    if not args.no_mixed:
        def form(prec):
            ms_p, tan_p, rec_p, launches_p = timed(prec)
            gbs = TANGENT32_BYTES_PER_ELEM * ne / (tan_p * 1e-3) / 1e9
            return {"value": ne / (ms_p * 1e-3), "ms_per_step": ms_p, "tangent_ms": tan_p, "recovery_ms": rec_p,
                    "speedup_vs_fp64": ms64 / ms_p, "tangent_hbm_gbs": gbs,
                    "tangent_hbm_frac": gbs / hbm if hbm else None, "gpu_launches": launches_p}
        fp32 = form(abi.TANGENT_FP32)
        # tensor-core forms of the same tangent (tcgen05.mma), one
        # Newton iteration each (tangent + FP64 recovery)
        tcf = {name: form(prec) for name, prec in TC_FORMS}
        head = tcf[HEADLINE_FORM]
        mixed = {"value": head["value"], "ms_per_step": head["ms_per_step"], "tangent_ms": head["tangent_ms"],
                 "recovery_ms": head["recovery_ms"], "speedup_vs_fp64": head["speedup_vs_fp64"],
                 "form": HEADLINE_FORM,
                 "dtype": f"tangent {HEADLINE_FORM} on the tensor cores (tcgen05.mma, FP32 accumulation), "
                          "recovery fp64",
                 "fp32": fp32, "tensor_core": tcf}
        eng.set_precision(abi.TANGENT_FP64)

    # whole-job throughput: max time over ranks
    value, t_step = whole_job_throughput(ne, ms64, world, dist, dev)

    # parity of this workload against the oracle: 64 blocks spread over the
    # mesh, one iteration from the same state; precision forms' Ke against
    # the oracle's FP64 Ke on the same blocks
    parity1 = None
    if not args.no_parity and rank == 0:
        forms = (("fp32", abi.TANGENT_FP32), ("tf32", abi.TANGENT_TF32), ("bf16", abi.TANGENT_BF16),
                 ("tf32x3", abi.TANGENT_TF32X3), ("bf16x3", abi.TANGENT_BF16X3))
        parity1 = parity_sample(eng, model, spread_blocks(model, 64), 2, 1, False, model.c, u1, du,
                                (tc.data_ptr(), tu.data_ptr(), tdu.data_ptr(), tifv.data_ptr()), stream,
                                precisions=forms)
    pins = regression_pins() if not args.no_parity and rank == 0 else None

    # ---- e2e through the host-array C-ABI ----
    e2e = None
    if not args.no_e2e:
        pin = lambda a: torch.from_numpy(a).pin_memory().numpy()
        c_h, u_h, du_h = pin(model.c), pin(u1), pin(du)
        ifv_p = pin(np.zeros(model.nodof))
        # all blocks' Ke back to back in one pinned buffer (estiff_blocks(blk)%ptr
        # would point into it)
        est_all = torch.empty(ne * model.utsz, dtype=torch.float64).pin_memory().numpy()
        for _ in range(2):
            eng.tanstf(2, 1, c_h, u_h, du_h, est_all)
            eng.recover(2, 1, False, c_h, u_h, du_h, ifv_p)
        barrier()
        reps = max(3, args.steps // 4)
        t0 = time.perf_counter()
        for _ in range(reps):
            eng.tanstf(2, 1, c_h, u_h, du_h, est_all)
            eng.recover(2, 1, False, c_h, u_h, du_h, ifv_p)
        t_e2e = (time.perf_counter() - t0) / reps
        h2d = 2 * 8 * (model.ncoord + 2 * model.nodof)
        d2h = 8 * (ne * model.utsz + model.nodof) + C.sizeof(abi.RecoverInfo)
        e2e = {"value": world * ne / t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": 1e3 * t_e2e, "estiff_to_host": True}

    solver = None
    if not args.no_solver:
        eng.set_precision(abi.TANGENT_FP64)
        solver = bench_solver(args, eng, model, tc, tu, tdu, dev)

    # ---- roofline of the dominant kernel ----
    traffic = load_traffic()
    if tan64 >= rec64:
        kname, kms, flop = "k_tangent_hex8<double>", tan64, TANGENT_FLOP_PER_ELEM
        tr = traffic.get("tangent_fp64_bytes_per_elem")
    else:
        kname, kms, flop = "k_recover_hex8", rec64, RECOVER_FLOP_PER_ELEM
        tr = traffic.get("recover_bytes_per_elem")
    achieved = flop * ne / (kms * 1e-3) / 1e12
    roofline = {"bound": "fp64", "kernel": kname, "achieved": achieved, "peak": fp64_peak_tflops,
                "unit": "TFLOP/s", "frac": achieved / fp64_peak_tflops,
                "traffic": (tr * ne) if tr else None,
                "peak_source": "measured live: w3g_measure_fp64_peak (DFMA chains, all SMs)",
                "algorithmic_flop_per_elem": flop,
                "tangent": {"ms": tan64, "tflops": TANGENT_FLOP_PER_ELEM * ne / (tan64 * 1e-3) / 1e12,
                            "tflops_refdense_count": TANGENT_FLOP_PER_ELEM_REFDENSE * ne / (tan64 * 1e-3) / 1e12,
                            "hbm_gbs": TANGENT_BYTES_PER_ELEM * ne / (tan64 * 1e-3) / 1e9},
                "recovery": {"ms": rec64, "tflops": RECOVER_FLOP_PER_ELEM * ne / (rec64 * 1e-3) / 1e12,
                             "tflops_refdense_count": RECOVER_FLOP_PER_ELEM_REFDENSE * ne / (rec64 * 1e-3) / 1e12,
                             "hbm_gbs": RECOVER_BYTES_PER_ELEM * ne / (rec64 * 1e-3) / 1e9}}
    roofline["hbm_peak_gbs_measured"] = hbm_peak_gbs()

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.n, args.cpu_sample_blocks, host_threads())

    formulations = None
    if not args.no_formulations:
        formulations = bench_formulations(args, dev, local)

    crystal = None
    if not args.no_crystal:
        eng.close()
        torch.cuda.empty_cache()
        crystal = bench_crystal(args, dev, local, rank == 0 and not args.no_cpu_baseline)

    batched = None
    if not args.no_batched:
        eng.close()
        del tc, tu, tdu, tifv
        torch.cuda.empty_cache()
        batched = bench_batched(args, dev, local)

    if rank == 0:
        # the full record first, then the headline line (last line of the
        # output) with compact summaries of every leg
        details = {"details": {"mixed": mixed, "batched": batched, "crystal": crystal, "solver": solver,
                               "formulations": formulations, "parity_hex8_64cube": parity1, "warp3d_regression": pins, "roofline": roofline,
                               "cpu_baseline": cb, "e2e": e2e}}
        print(json.dumps(details), flush=True)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{args.n}^3 hex8 l3disop geonl (jitter 0.1h), mm01 bilinear, blocks of 128, "
                                   f"1 Newton iteration = tangent + recovery",
                       "elements": ne, "gauss_points": ne * 8, "l2": "inputs ~3 GB per step > L2, no flush",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
            "tangent_ms": tan64, "recovery_ms": rec64,
            "mixed": summarize_mixed(mixed), "e2e": e2e, "roofline": compact_roofline(roofline),
            "cpu_baseline": cb, "clocks": clocks, "gpu_launches": launches64,
            "parity": summarize_parity(parity1, batched, crystal, pins),
            "batched": summarize_leg(batched), "crystal": summarize_leg(crystal),
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
