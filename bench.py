"""Benchmark of the Osd evaluation hot path on GB300 (one JSON line on stdout).

Workload (one "step" = one pass of the hot path over one batch): the plain-method torus --
512 x 256 quads, 5% split into triangles, 2% semi-sharp creases, Catmull-Clark uniform level 3
(8,598,400 factorized stencils, 112M entries), 8 interleaved float32 primvars -- EvalStencils
over every level-3 point, then limit EvalStencils (P, du, dv fused) at 1M seeded locations.
Metric: stencil evaluations per second (refined + limit points per step / step time).

  value  -- tables, source and outputs resident in HBM, CUDA events on the launch stream;
  e2e    -- through the public C-ABI with host buffers: per step the deformed control points
            are copied from pinned host memory into the GB300 vertex buffer, both evaluations
            run, and all outputs are copied back to pinned host memory (steps pipelined: a
            step's evaluation overlaps the previous step's readback).
The per-step working set (1.4 GB of tables and outputs) exceeds the 129 MB L2, so no
explicit flush is needed between steps.

--impl reference times the CPU evaluator of the path on this host's cores (the oracle port
of Osd::CpuEvaluator / OmpEvaluator; the reference's C++ library is compiled for the build
host only) on the same workload, one bounded sample per step, and adds `reference_cuda`: the
reference's own CUDA evaluator kernels (osd/cudaKernel.cu, compiled for sm_103a by the oracle
recipe) launched with its own launch logic on the same GPU and workloads.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--nu", type=int, default=512, help="torus cage resolution (u)")
    ap.add_argument("--nv", type=int, default=256, help="torus cage resolution (v)")
    ap.add_argument("--n-limit", type=int, default=1_000_000, help="limit locations")
    ap.add_argument("--no-patches", action="store_true", help="skip the EvalPatches section")
    ap.add_argument("--no-config1", action="store_true",
                    help="skip the CPU-runnable cube section (warm and cold L2)")
    ap.add_argument("--patch-points", type=int, default=4_000_000)
    ap.add_argument("--no-bfr", action="store_true",
                    help="skip the Bfr tessellate-and-evaluate section")
    ap.add_argument("--no-batch", action="store_true", help="skip the batching section")
    ap.add_argument("--batch-meshes", type=int, default=256)
    ap.add_argument("--batch-cv-max", type=int, default=200_000,
                    help="upper end of the log-uniform CV range of the batched meshes")
    ap.add_argument("--batch-cv-max-scaled", type=int, default=25_000,
                    help="also run a population with this smaller CV range (0: skip)")
    ap.add_argument("--serve-cv-max", type=int, default=25_000,
                    help="upper end of the CV range of the serving pool's topologies")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving section")
    ap.add_argument("--no-factory", action="store_true",
                    help="skip the stencil-table factory section")
    ap.add_argument("--layouts", action="store_true",
                    help="add the `layouts` section: device-table EvalStencils per primvar "
                         "layout (L = 3/4/8/12) and per output count (1-6)")
    ap.add_argument("--serve-topologies", type=int, default=1000)
    ap.add_argument("--serve-requests", type=int, default=4000, help="requests per rate")
    ap.add_argument("--serve-rates", type=lambda s: [float(x) for x in s.split(",")],
                    default=[2000.0, 5000.0, 10000.0, 20000.0])
    ap.add_argument("--serve-budget-gb", type=float, default=40.0)
    ap.add_argument("--serve-ring-mb", type=int, default=4096,
                    help="pinned host ring for request outputs")
    return ap.parse_args()


GOLDEN = os.path.join(ROOT, "tests", "golden")
# the EvalPatches tables: the reference's own adaptive level-4 tables of the full-size cages
# (written by tests/golden/make_golden.py large where the reference is available) or, when
# they are absent, stand-ins of their size instanced from the small fixtures
PATCH_TABLES = {
    False: ("torus512x256_adaptiveL4.npz", "torus512x256_adaptiveL4_gregory",
            "torus32x16_patches_L4.npz", 1_431_592, None, 7),
    True: ("icosphere6_loop_adaptiveL4.npz", "icosphere6_loop_adaptiveL4",
           "icosphere2_patches_L3.npz", 82_580, 5, 8),
}


def host_link_gbs(nbytes=1 << 30, reps=5):
    """Pinned host <-> device copy bandwidth right now (GB/s, median of `reps`, CUDA events)."""
    import torch
    h = torch.empty(nbytes // 4, pin_memory=True)
    d = torch.empty(nbytes // 4, device="cuda")
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        out[name] = nbytes / (float(np.median(ms)) / 1e3) / 1e9
    del h, d
    return out


def release_memory():
    """Frees what a finished section left behind: Python objects (tables, buffers) and the
    blocks torch's caching allocator keeps."""
    import gc

    import torch
    gc.collect()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def fp32_rate(stream):
    """Measured FP32 FMA rate of this GPU in TFLOP/s (GB300MeasureFp32Rate, once per run)."""
    global _FP32
    if _FP32 is None:
        import ctypes

        from opensubdiv_gb300 import _lib
        v = ctypes.c_double(0.0)
        _lib.check(_lib.load().GB300MeasureFp32Rate(ctypes.byref(v),
                                                      ctypes.c_void_p(stream.cuda_stream)))
        _FP32 = v.value
    return _FP32


_FP32 = None


def patch_workload(n_points, loop=False):
    from opensubdiv_gb300 import workloads
    large, name, small, target, count_type, seed = PATCH_TABLES[loop]
    path = os.path.join(GOLDEN, "large", large)
    if os.path.exists(path):
        w = workloads.eval_patches_points(np.load(path), name, n_points, seed)
        w["table_source"] = "the reference's own Far::PatchTableFactory table of the cage"
        return w
    w = workloads.instanced_points(np.load(os.path.join(GOLDEN, small)),
                                   "standin_" + small[:-4], target, n_points, seed, count_type)
    w["table_source"] = (f"stand-in: {small} instanced {w['copies']}x to the full table's "
                         "size (the full-size table was not generated where build() ran)")
    return w


def serving_bases():
    from opensubdiv_gb300 import shapes, workloads
    return {shapes.CATMARK: workloads.ServingBase(
                np.load(os.path.join(GOLDEN, "torus32x16_patches_L4.npz"))),
            shapes.LOOP: workloads.ServingBase(
                np.load(os.path.join(GOLDEN, "icosphere2_patches_L3.npz")))}


def bench_patches(args, stream, peak, loop=False):
    """Secondary measurement: device PatchMap lookup + EvalPatches (P and all five
    derivatives) at 4M uniform points on the 512 x 256 torus's adaptive level-4 table with
    Gregory-basis end caps or, with `loop`, the level-6 icosphere's adaptive Loop table
    (patch_workload)."""
    import torch

    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300PatchTable)

    w = patch_workload(args.patch_points, loop)
    n = len(w["face"])
    table = GB300PatchTable.Create(w["arrays"], w["indices"], w["params"], w["triangular"])
    src = torch.from_numpy(w["src"]).cuda()
    face = torch.from_numpy(w["face"]).cuda()
    u = torch.from_numpy(w["u"]).cuda()
    v = torch.from_numpy(w["v"]).cuda()
    coords = torch.empty(n * 5, dtype=torch.int32, device="cuda")
    outs = [torch.empty(n * 3, device="cuda") for _ in range(6)]
    d = BD(0, 3, 3)

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        table.FindPatches(n, face, u, v, coords, stream=stream)
        if ev:
            ev[1].record(stream)
        ok = Ev.EvalPatchesTable(src, d, outs[0], d, n, coords, table, du=outs[1], duDesc=d,
                                 dv=outs[2], dvDesc=d, duu=outs[3], duuDesc=d, duv=outs[4],
                                 duvDesc=d, dvv=outs[5], dvvDesc=d, stream=stream)
        assert ok
        if ev:
            ev[2].record(stream)

    fp32_peak = fp32_rate(stream)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    evs = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3))
           for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            step(evs[k])
    torch.cuda.synchronize()
    find_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
    eval_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in evs]))
    ch_all = coords.view(n, 5).cpu().numpy()
    c = ch_all[:, 1]
    touched = int(len(np.unique(c[c >= 0])))
    cvs = float(np.average(w["arrays"][:, 4], weights=w["arrays"][:, 2]))
    b = workloads.patch_bytes(n, 3, 6, len(w["src"]) // 3, touched, cvs)
    types = workloads.point_types(ch_all, w["arrays"], w["params"])
    flops = workloads.patch_flops(types, 3)
    gathered = workloads.patch_gathered_bytes(types, 3, 6)
    # spot check against the oracle on a slice (outside timing)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    k = 20000
    ch = coords[: k * 5].view(k, 5).cpu().numpy()
    ref = [np.zeros(k * 3, np.float32) for _ in range(6)]
    oracle.eval_patches(w["src"], (0, 3, 3), ref, [(0, 3, 3)] * 6, ch, w["arrays"],
                        w["indices"], w["params"], threads=8)
    err_p = float(np.abs(outs[0][: k * 3].cpu().numpy() - ref[0]).max())
    return {"workload": w["name"], "table": w["table_source"], "points": n,
            "patch_arrays": w["arrays"].tolist(), "source_points": len(w["src"]) // 3, "patch_evals_per_s": n / ((find_ms + eval_ms) / 1e3),
            "find_patches_ms": find_ms, "eval_patches_ms": eval_ms, "outputs": 6,
            "patches_touched": touched,
            "roofline": {"bound": "hbm", "kernel": "k_eval_patches (P + 5 derivatives)",
                         "algorithmic_bytes": b, "achieved": b / (eval_ms / 1e3) / 1e9,
                         "peak": peak, "unit": "GB/s",
                         "frac": b / (eval_ms / 1e3) / 1e9 / peak,
                         "traffic": ncu_traffic("patches_loop" if loop else "patches"),
                         "as_gathered_bytes": gathered,
                         "as_gathered_gbs": gathered / (eval_ms / 1e3) / 1e9,
                         "fp32": {"flops_per_launch": flops,
                                  "achieved_tflops": flops / (eval_ms / 1e3) / 1e12,
                                  "peak_tflops": fp32_peak,
                                  "frac": flops / (eval_ms / 1e3) / 1e12 / fp32_peak,
                                  "peak_kind": "measured (GB300MeasureFp32Rate)"},
                         "point_types": {str(t): int((types == t).sum())
                                         for t in np.unique(types)}},
            "max_abs_err_P_vs_oracle_slice": err_p}


BFR_TABLE = "torus512x256_bfr.npz"
BFR_INTERVAL = 0.0022  # edge-length interval of the non-uniform rates (mean rate ~5.1)


def bench_bfr(args, stream, peak):
    """Bfr tessellate-and-evaluate of every face of the 512 x 256 torus in one pass (the loop
    the reference's Bfr tutorials run face by face, tutorials/bfr/tutorial_1_2 and 2_1):
    GB300TessellationCount + GB300TessellationGenerate (coords, triangle facets with mesh-wide
    indices, PatchCoords located on the Far table of Bfr::SurfaceFactory's default
    approximation) + GB300TessellationEvaluate of P, Du and Dv (and, for comparison, the same
    points through the general GB300PatchTableEval).  Two rate schemes: the tutorials'
    uniform rate 5, and per-edge rates from control-hull edge lengths (tutorial 2.1)."""
    import torch

    from opensubdiv_gb300 import bfr, workloads
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300PatchTable)

    path = os.path.join(GOLDEN, "large", BFR_TABLE)
    if not os.path.exists(path):
        return {"skipped": f"{BFR_TABLE} is written where the reference is available "
                           "(tests/golden/make_golden.py large)"}
    z = np.load(path)
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"], False)
    src = torch.from_numpy(z["src"]).cuda()
    sizes_host = np.ascontiguousarray(z["verts_per_face"], np.int32)
    nfaces = len(sizes_host)
    d = BD(0, 3, 3)
    cvs = float(np.average(z["arrays"][:, 4], weights=z["arrays"][:, 2]))

    def touched_patches(patch_coords):
        return int(len(np.unique(patch_coords[:, 1].cpu().numpy())))

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    out = {"workload": "torus512x256 (5% triangles, 2% creases), Bfr::SurfaceFactory default "
                       "approximation (sharp 6 / smooth 2) as a Far table",
           "faces": nfaces, "patches": int(len(z["params"])), "facet_size": 3,
           "outputs": "P, Du, Dv"}
    for mode in ("uniform5", "edge_lengths"):
        if mode == "uniform5":
            kw = dict(uniform_rate=5)
            rate_desc = "uniform rate 5"
        else:
            ro, rates = workloads.bfr_edge_length_rates(z["positions"], z["verts_per_face"],
                                                        z["face_verts"], BFR_INTERVAL)
            kw = dict(rates=rates, rate_offsets=ro)
            rate_desc = (f"edge rates 1 + int(hull length / {BFR_INTERVAL}) (mean {rates.mean():.2f}, "
                         f"{rates.min()}..{rates.max()})")
        m = bfr.MeshTessellation(4, sizes_host, options=bfr.TessellationOptions(3), stream=stream,
                                 **kw)
        n, nf = m.num_coords, m.num_facets
        coords = torch.empty((n, 2), device="cuda")
        facets = torch.empty((nf, 3), dtype=torch.int32, device="cuda")
        pc = torch.empty((n, 5), dtype=torch.int32, device="cuda")
        outs = [torch.empty(n * 3, device="cuda") for _ in range(3)]

        def gen():
            m.Generate(coords, facets, True, table, pc)

        def ev():
            m.Evaluate(src, d, table, pc, 1, outs)

        def ev_table():
            assert Ev.EvalPatchesTable(src, d, outs[0], d, n, pc, table, du=outs[1], duDesc=d,
                                       dv=outs[2], dvDesc=d, stream=stream)

        for _ in range(args.warmup):
            gen()
            ev()
        torch.cuda.synchronize()
        evs = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3))
               for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                evs[k][0].record(stream)
                gen()
                evs[k][1].record(stream)
                ev()
                evs[k][2].record(stream)
        torch.cuda.synchronize()
        gen_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in evs]))
        eval_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in evs]))
        # the same points through the general EvalPatches entry (element-lane kernel)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            ev_table()
            e0.record(stream)
            for _ in range(args.steps):
                ev_table()
            e1.record(stream)
        torch.cuda.synchronize()
        eval_table_ms = e0.elapsed_time(e1) / args.steps
        # Count waits for its totals: timed on the host
        t0 = time.perf_counter()
        for _ in range(args.steps):
            m.Count()
        count_ms = (time.perf_counter() - t0) * 1e3 / args.steps

        # end to end from host buffers: face sizes and rates in, P / Du / Dv, coords and facets
        # out (the control points' patch points stay resident, as the tutorial's mesh does)
        h_sizes = torch.from_numpy(sizes_host).pin_memory()
        h_rates = (torch.from_numpy(np.concatenate([kw["rate_offsets"], kw["rates"]]))
                   .pin_memory() if "rates" in kw else None)
        h_out = [torch.empty(n * 3, pin_memory=True) for _ in range(3)]
        h_coords = torch.empty((n, 2), pin_memory=True)
        h_facets = torch.empty((nf, 3), dtype=torch.int32, pin_memory=True)

        def e2e():
            with torch.cuda.stream(stream):
                dsz = h_sizes.to("cuda", non_blocking=True)
                mk = dict(uniform_rate=5)
                if h_rates is not None:
                    dr = h_rates.to("cuda", non_blocking=True)
                    mk = dict(rate_offsets=dr[:nfaces + 1], rates=dr[nfaces + 1:])
                mm = bfr.MeshTessellation(4, dsz, options=bfr.TessellationOptions(3),
                                          stream=stream, **mk)
                mm.Generate(coords, facets, True, table, pc)
                mm.Evaluate(src, d, table, pc, 1, outs)
                for a, b in zip(h_out, outs):
                    a.copy_(b, non_blocking=True)
                h_coords.copy_(coords, non_blocking=True)
                h_facets.copy_(facets, non_blocking=True)
            stream.synchronize()

        for _ in range(2):
            e2e()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        h2d = 4 * nfaces + (4 * (nfaces + 1 + len(kw["rates"])) if "rates" in kw else 0)
        d2h = 36 * n + 8 * n + 12 * nf

        # correctness (outside timing): every coord and facet of the mesh bit for bit against
        # the oracle, and P / Du / Dv on a slice against the oracle's evaluation
        tm = oracle.tess_mesh(4, sizes_host, kw.get("rate_offsets", np.arange(nfaces + 1)),
                              kw.get("rates", np.full(nfaces, 5, np.int32)), 3, False, threads=16)
        exact = bool(np.array_equal(h_coords.numpy().view(np.int32),
                                    tm["coords"].view(np.int32)) and
                     np.array_equal(h_facets.numpy(), tm["facets"]))
        k = min(n, 200_000)
        pch = pc[:k].cpu().numpy()
        ref = [np.zeros(k * 3, np.float32) for _ in range(3)]
        oracle.eval_patches(z["src"], (0, 3, 3), ref, [(0, 3, 3)] * 3, pch, z["arrays"],
                            z["patch_indices"], z["params"], threads=16)
        err = max(float(np.abs(h_out[j].numpy()[: k * 3] - ref[j]).max()) for j in range(3))

        # shared (watertight) points, the reference's tutorial 2.2: Share on a fresh copy of the
        # facets each step (the call reads the point total back), then each point evaluated
        # once; end to end from host buffers with the face vertices and edges uploaded too
        fe_host, n_edges = workloads.face_edges(z["verts_per_face"], z["face_verts"])
        fv_host = np.ascontiguousarray(z["face_verts"], np.int32)
        n_verts = len(z["positions"])
        fv_dev = torch.from_numpy(fv_host).cuda()
        fe_dev = torch.from_numpy(fe_host).cuda()
        gen()
        facets_coord = facets.clone()
        sh_facets = torch.empty_like(facets)
        pts = None
        for _ in range(args.warmup):
            sh_facets.copy_(facets_coord)
            pts = m.Share(fv_dev, fe_dev, n_verts, n_edges, sh_facets, patch_coords=pc)
        np_ = pts.num_points
        pouts = [torch.empty(np_ * 3, device="cuda") for _ in range(3)]
        share_ms, peval_ms = [], []
        for _ in range(args.steps):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            with torch.cuda.stream(stream):
                sh_facets.copy_(facets_coord)
                e0.record(stream)
                pts = m.Share(fv_dev, fe_dev, n_verts, n_edges, sh_facets, patch_coords=pc,
                              out=pts)
                e1.record(stream)
                m.Evaluate(src, d, table, pts.patch_coords, 1, pouts, num_points=np_)
                e2.record(stream)
            torch.cuda.synchronize()
            share_ms.append(e0.elapsed_time(e1))
            peval_ms.append(e1.elapsed_time(e2))
        share_ms, peval_ms = float(np.median(share_ms)), float(np.median(peval_ms))
        h_fv = torch.from_numpy(fv_host).pin_memory()
        h_fe = torch.from_numpy(fe_host).pin_memory()
        h_pout = [torch.empty(np_ * 3, pin_memory=True) for _ in range(3)]

        def e2e_shared():
            with torch.cuda.stream(stream):
                dsz = h_sizes.to("cuda", non_blocking=True)
                dfv = h_fv.to("cuda", non_blocking=True)
                dfe = h_fe.to("cuda", non_blocking=True)
                mk = dict(uniform_rate=5)
                if h_rates is not None:
                    dr = h_rates.to("cuda", non_blocking=True)
                    mk = dict(rate_offsets=dr[:nfaces + 1], rates=dr[nfaces + 1:])
                mm = bfr.MeshTessellation(4, dsz, options=bfr.TessellationOptions(3),
                                          stream=stream, **mk)
                mm.Generate(coords, facets, True, table, pc)
                sp = mm.Share(dfv, dfe, n_verts, n_edges, facets, patch_coords=pc)
                mm.Evaluate(src, d, table, sp.patch_coords, 1, pouts, num_points=sp.num_points)
                for a, b in zip(h_pout, pouts):
                    a.copy_(b, non_blocking=True)
                h_facets.copy_(facets, non_blocking=True)
            stream.synchronize()

        for _ in range(2):
            e2e_shared()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_shared()
        e2e_sh_ms = (time.perf_counter() - t0) * 1e3 / args.steps
        h2d_sh = h2d + 8 * len(fv_host)
        d2h_sh = 36 * np_ + 12 * nf
        # outside timing: the watertight facets and point numbering against the oracle's
        # bookkeeping (exact), the points' P against the per-coord evaluation
        w_f, w_po, w_src = oracle.tess_share(4, sizes_host, fv_host, fe_host, n_verts, n_edges,
                                             kw.get("rate_offsets", np.arange(nfaces + 1)),
                                             kw.get("rates", np.full(nfaces, 5, np.int32)),
                                             tm["coord_offsets"], tm["facet_offsets"],
                                             tm["facets"])
        shared_exact = bool(np_ == len(w_src) and np.array_equal(h_facets.numpy(), w_f))
        pp = h_pout[0].numpy().reshape(-1, 3)
        shared_p_bitwise = bool(np.array_equal(pp.view(np.int32),
                                               h_out[0].numpy().reshape(-1, 3)[w_src]
                                               .view(np.int32)))
        share_b = workloads.bfr_share_bytes(nfaces, len(fv_host), n_verts, n_edges, nf, np_, 3)
        peval_b = workloads.patch_bytes(np_, 3, 3, len(z["src"]) // 3, touched_patches(pc), cvs)
        shared = {
            "points": np_, "points_per_coord": np_ / n,
            "share_ms": share_ms, "eval_points_ms": peval_ms,
            "points_per_s": np_ / ((gen_ms + share_ms + peval_ms) / 1e3),
            "e2e": {"points_per_s": np_ / (e2e_sh_ms / 1e3), "ms": e2e_sh_ms,
                    "h2d_bytes": h2d_sh, "d2h_bytes": d2h_sh,
                    "what": "host face sizes (and rates), face vertices and edges in; Count, "
                            "Generate, Share, Eval of each point once; P/Du/Dv of the points "
                            "and the facets back to pinned host memory"},
            "roofline_share": {"bound": "hbm", "kernel": "k_share_* (7 launches + 2 scans)",
                               "algorithmic_bytes": share_b,
                               "achieved": share_b / (share_ms / 1e3) / 1e9, "peak": peak,
                               "unit": "GB/s", "frac": share_b / (share_ms / 1e3) / 1e9 / peak,
                               "note": "share_ms is the whole call, including its host read of "
                                       "the point total",
                               "traffic_emit": ncu_traffic("bfr_share_emit")},
            "roofline_eval": {"bound": "hbm", "algorithmic_bytes": peval_b,
                              "achieved": peval_b / (peval_ms / 1e3) / 1e9, "peak": peak,
                              "unit": "GB/s", "frac": peval_b / (peval_ms / 1e3) / 1e9 / peak},
            "exact_facets_and_points_vs_oracle": shared_exact,
            "points_p_bitwise_vs_per_coord_eval": shared_p_bitwise,
        }
        del fv_dev, fe_dev, facets_coord, sh_facets, pouts, h_pout, pts

        # CPU baseline: the oracle's tessellate + locate + evaluate over a bounded face sample
        sample = max(1, nfaces // 8)
        so = np.concatenate([[0], np.cumsum(np.ones(sample, np.int64))]) if "rates" not in kw \
            else None
        cpu_threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        if "rates" in kw:
            r_off = kw["rate_offsets"][: sample + 1]
            r_sel = kw["rates"][: r_off[-1]]
        else:
            r_off = so.astype(np.int32)
            r_sel = np.full(sample, 5, np.int32)
        ct = oracle.tess_mesh(4, sizes_host[:sample], r_off, r_sel, 3, False, threads=cpu_threads)
        ptex = np.concatenate([[0], np.cumsum(np.where(sizes_host[:sample] == 4, 1,
                                                       sizes_host[:sample]))])
        qf, st = oracle.tess_locate_mesh(4, sizes_host[:sample], ct["coord_offsets"], ptex,
                                         ct["coords"], threads=cpu_threads)
        pm = oracle.PatchMap(z["arrays"], z["params"], False)
        hh = pm.find(qf, st[:, 0].astype(np.float64), st[:, 1].astype(np.float64))
        cc = oracle.make_coords(hh, st[:, 0], st[:, 1])
        co3 = [np.zeros(len(cc) * 3, np.float32) for _ in range(3)]
        oracle.eval_patches(z["src"], (0, 3, 3), co3, [(0, 3, 3)] * 3, cc, z["arrays"],
                            z["patch_indices"], z["params"], threads=cpu_threads)
        cpu_s = time.perf_counter() - t0

        facet_b = workloads.bfr_tess_bytes(nfaces, n, nf, 3, True, "rates" not in kw)
        eval_b = workloads.patch_bytes(n, 3, 3, len(z["src"]) // 3, touched_patches(pc), cvs)
        out[mode] = {
            "rates": rate_desc, "coords": n, "facets": nf,
            "points_per_s": n / ((gen_ms + eval_ms) / 1e3),
            "tessellate_ms": gen_ms, "eval_ms": eval_ms, "count_ms_host": count_ms,
            "eval_ms_general_entry": eval_table_ms,
            "e2e": {"points_per_s": n / (e2e_ms / 1e3), "ms": e2e_ms, "h2d_bytes": h2d,
                    "d2h_bytes": d2h,
                    "what": "host face sizes (and rates) in; Count, Generate, Eval; P/Du/Dv, "
                            "coords and facets back to pinned host memory"},
            "roofline_tessellate": {"bound": "hbm", "kernel": "k_tess_generate + k_tess_finish",
                                    "algorithmic_bytes": facet_b,
                                    "achieved": facet_b / (gen_ms / 1e3) / 1e9, "peak": peak,
                                    "unit": "GB/s",
                                    "frac": facet_b / (gen_ms / 1e3) / 1e9 / peak,
                                    "traffic": ncu_traffic("bfr_" + mode)},
            "roofline_eval": {"bound": "hbm", "kernel": "k_eval_patches<3, 1> (P, Du, Dv; GB300TessellationEvaluate)",
                              "algorithmic_bytes": eval_b,
                              "achieved": eval_b / (eval_ms / 1e3) / 1e9, "peak": peak,
                              "unit": "GB/s", "frac": eval_b / (eval_ms / 1e3) / 1e9 / peak},
            "exact_coords_and_facets_vs_oracle": exact,
            "max_abs_err_vs_oracle_slice": err,
            "shared_points": shared,
            "cpu_baseline": {"value": len(cc) / cpu_s, "unit": "points/s", "cores": cpu_threads,
                             "kind": "port",
                             "sample": f"first {sample} faces ({len(cc)} points): oracle "
                                       "tessellate + locate + PatchMap + EvalPatches"},
        }
        del m, coords, facets, pc, outs
        release_memory()

    # draw-time tessellation factors of every patch of the table (screen-space, camera framing
    # the torus, fractional-odd spacing): the patch shaders' tess-control math
    from opensubdiv_gb300.evaluator import PatchTessOptions
    npatch = int(len(z["params"]))
    p = np.asarray(z["positions"], np.float64)
    c, r = 0.5 * (p.min(0) + p.max(0)), float(np.linalg.norm(p.max(0) - p.min(0)))
    eye = c + np.array([0.3, 0.4, 1.0]) * r
    f = (c - eye) / np.linalg.norm(c - eye)
    sx = np.cross(f, [0.0, 1.0, 0.0])
    sx /= np.linalg.norm(sx)
    ux = np.cross(sx, f)
    mv = np.eye(4)
    mv[0, :3], mv[1, :3], mv[2, :3] = sx, ux, -f
    mv[:3, 3] = -mv[:3, :3] @ eye
    near, far = 0.01 * r, 10.0 * r
    pr = np.zeros((4, 4))
    pr[0, 0] = pr[1, 1] = 1.0 / np.tan(np.radians(22.5))
    pr[2, 2], pr[2, 3], pr[3, 2] = (far + near) / (near - far), 2 * far * near / (near - far), -1
    to = PatchTessOptions(24.0, 64.0, True, 2, mv, pr)
    tf = [torch.empty((npatch, 4), device="cuda"), torch.empty((npatch, 2), device="cuda"),
          torch.empty((npatch, 4), device="cuda"), torch.empty((npatch, 4), device="cuda")]
    for _ in range(args.warmup):
        table.TessFactors(to, *tf, src=src, stream=stream)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        t0.record(stream)
        for _ in range(args.steps):
            table.TessFactors(to, *tf, src=src, stream=stream)
        t1.record(stream)
    torch.cuda.synchronize()
    tf_ms = t0.elapsed_time(t1) / args.steps
    out["tess_factors"] = {"patches": npatch, "ms": tf_ms, "patches_per_s": npatch / (tf_ms / 1e3),
                           "mode": "screen-space, fractional-odd spacing, tess level 24"}
    del table, src
    release_memory()
    out["limit_stencils"] = bench_bfr_stencils(args, stream, peak)
    return out


BFR_STENCIL_TABLE = "torus256x128_bfr_stencils.npz"


def bench_bfr_stencils(args, stream, peak):
    """Bfr::Surface::EvaluateStencil at every tessellation point (GB300TessellationStencils) on
    the 256 x 128 torus at rate 5, and the two per-frame paths it enables: (a) EvalStencils of
    the points straight from the cage with those stencils, against (b) refining the patch
    points from the cage with Far's point stencils, then GB300TessellationEvaluate.  Each frame
    evaluates P, Du and Dv of every point."""
    import torch

    from opensubdiv_gb300 import bfr, workloads
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300PatchTable, GB300StencilTable)

    path = os.path.join(GOLDEN, "large", BFR_STENCIL_TABLE)
    if not os.path.exists(path):
        return {"skipped": f"{BFR_STENCIL_TABLE} is written where the reference is available "
                           "(tests/golden/make_golden.py large)"}
    z = np.load(path)
    pos = np.ascontiguousarray(z["positions"], np.float32)
    nc = len(pos)
    table = GB300PatchTable.Create(z["arrays"], z["patch_indices"], z["params"], False)
    m = bfr.MeshTessellation(4, z["verts_per_face"], uniform_rate=5,
                             options=bfr.TessellationOptions(3), stream=stream)
    _, _, pc = m.Generate(table=table)
    n = m.num_coords
    st_sizes, st_offsets = z["st_sizes"], z["st_offsets"]
    st_indices, st_weights = z["st_indices"], z["st_weights"]
    base = GB300StencilTable.Create(
        np.concatenate([np.ones(nc, np.int32), st_sizes]),
        np.concatenate([np.arange(nc), nc + st_offsets]),
        np.concatenate([np.arange(nc), st_indices]),
        np.concatenate([np.ones(nc, np.float32), st_weights]))
    refine = GB300StencilTable.Create(st_sizes, st_offsets, st_indices, st_weights)
    setup = []
    lim = None
    for _ in range(max(args.warmup, 3)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lim = GB300StencilTable.FromPatchCoords(table, pc, base, channels=3, stream=stream)
        torch.cuda.synchronize()
        setup.append((time.perf_counter() - t0) * 1e3)
    nnz = lim.GetNumIndices()
    d = BD(0, 3, 3)
    cage = torch.from_numpy(pos.ravel()).cuda()
    srcbuf = torch.zeros(len(z["src"]), device="cuda")
    srcbuf[: nc * 3] = cage
    a_out = [torch.empty(n * 3, device="cuda") for _ in range(3)]
    b_out = [torch.empty(n * 3, device="cuda") for _ in range(3)]

    def path_a():
        Ev.EvalStencilsTable(cage, d, a_out[0], d, lim, du=a_out[1], duDesc=d, dv=a_out[2],
                             dvDesc=d, stream=stream)

    def path_b():
        Ev.EvalStencilsTable(srcbuf, d, srcbuf, BD(nc * 3, 3, 3), refine, stream=stream)
        m.Evaluate(srcbuf, d, table, pc, 1, b_out)

    res = {}
    for name, fn in (("stencils_from_cage", path_a), ("refine_then_patches", path_b)):
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for e0, e1 in ev:
                e0.record(stream)
                fn()
                e1.record(stream)
        torch.cuda.synchronize()
        res[name] = float(np.median([e0.elapsed_time(e1) for e0, e1 in ev]))
    diag = float(np.linalg.norm(pos.max(0).astype(np.float64) - pos.min(0)))
    err = max(float((a - b).abs().max()) for a, b in zip(a_out, b_out))
    sb = workloads.stencil_bytes(n, nnz, 3, nc, n_weight_arrays=3, n_outputs=3)
    return {
        "workload": "torus256x128 (5% triangles, 2% creases), uniform rate 5, P/Du/Dv, "
                    "Bfr::SurfaceFactory default approximation as a Far table",
        "faces": int(len(z["verts_per_face"])), "points": n, "stencil_entries": int(nnz),
        "setup_ms_host": float(np.median(setup)),
        "frame_ms": res,
        "frame_points_per_s": {k: n / (v / 1e3) for k, v in res.items()},
        "roofline_stencils_from_cage": {
            "bound": "hbm", "kernel": "EvalStencils over the point stencils",
            "algorithmic_bytes": sb, "achieved": sb / (res["stencils_from_cage"] / 1e3) / 1e9,
            "peak": peak, "unit": "GB/s",
            "frac": sb / (res["stencils_from_cage"] / 1e3) / 1e9 / peak},
        "max_abs_diff_between_paths_rel_bbox_diag": err / diag,
    }


def bench_batch(args, stream, peak, cv_max):
    """Batching: a population of meshes of uneven size (workloads.batch_population_masks, CV
    counts log-uniform in [500, cv_max]) evaluated per frame as ONE persistent launch replayed
    from a CUDA graph (GB300StencilBatch, tuned), against one plain EvalStencilsTable call per
    mesh.  A frame = sinusoidal deformation of every control value (one elementwise pass over
    all meshes' sources, same in both arms) + evaluation of every mesh.  The tables are built
    on the device by the GPU stencil-table factory from host-recorded masks, mesh by mesh as
    the host threads produce them."""
    import torch

    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilBatch,
                                            GB300StencilTableFactory as Factory)

    t0 = time.time()
    pop, tables = [], []
    factory_s = 0.0
    for m in workloads.batch_population_masks(n_meshes=args.batch_meshes, cv_max=cv_max):
        nc, levels = m.pop("masks")
        t1 = time.time()
        tables.append(Factory.Create(nc, levels, generateIntermediateLevels=False))
        factory_s += time.time() - t1
        m["n_stencils"] = tables[-1].GetNumStencils()
        m["nnz"] = int(tables[-1].GetNumIndices())
        pop.append(m)
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    order = np.argsort([m["index"] for m in pop], kind="stable")  # population order
    pop = [pop[i] for i in order]
    tables = [tables[i] for i in order]
    # one concatenated source / base / phase buffer and one destination buffer, every mesh's
    # slice starting on a 32-byte boundary
    al = lambda x: (x + 7) // 8 * 8  # noqa: E731
    s_off, d_off, so, do = [], [], 0, 0
    for m in pop:
        s_off.append(so)
        d_off.append(do)
        so += al(m["n_cv"] * m["length"])
        do += al(m["n_stencils"] * m["length"])
    base_h = np.zeros(so, np.float32)
    phase_h = np.zeros(so, np.float32)
    for m, o in zip(pop, s_off):
        base_h[o:o + len(m["src"])] = m["src"]
        phase_h[o:o + len(m["src"])] = m["phase"]
    base = torch.from_numpy(base_h).cuda()
    phase = torch.from_numpy(phase_h).cuda()
    src = base.clone()
    dst = torch.zeros(do, device="cuda")
    descs = [BD(0, m["length"], m["length"]) for m in pop]
    sp = [src.data_ptr() + 4 * o for o in s_off]
    dp = [dst.data_ptr() + 4 * o for o in d_off]
    n_st = sum(m["n_stencils"] for m in pop)
    nnz = sum(m["nnz"] for m in pop)
    b_alg = sum(workloads.stencil_bytes(m["n_stencils"], m["nnz"], m["length"], m["n_cv"])
                for m in pop)
    batch = GB300StencilBatch(list(zip(tables, sp, descs, dp, descs)), stream=stream)
    with torch.cuda.stream(stream):
        batch.Tune(iterations=3, stream=stream)
    cfg = batch.GetConfig()

    def deform(frame):
        torch.add(base, torch.sin(0.1 * frame + phase + 7.0 * base), alpha=0.01, out=src)

    def plain_eval():
        for t, s, d, de in zip(tables, sp, dp, descs):
            assert Ev.EvalStencilsTable(s, de, d, de, t, stream=stream)

    def batched_eval():
        batch.EvalGraph(stream=stream)

    def run(fn):
        for f in range(args.warmup):
            deform(f)
            fn()
        torch.cuda.synchronize()
        ev = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3))
              for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for f in range(args.steps):
                ev[f][0].record(stream)
                deform(f)
                ev[f][1].record(stream)
                fn()
                ev[f][2].record(stream)
        torch.cuda.synchronize()
        frame = np.array([e[0].elapsed_time(e[2]) for e in ev])
        evals = np.array([e[1].elapsed_time(e[2]) for e in ev])
        return frame, evals

    with torch.cuda.stream(stream):
        fp, ep = run(plain_eval)
        deform(0)
        plain_eval()
        torch.cuda.synchronize()
        ref = dst.clone()
        dst.zero_()
        fb, eb = run(batched_eval)
        deform(0)
        batched_eval()
        torch.cuda.synchronize()
    identical = bool(torch.equal(dst, ref))
    del ref
    status = batch.GetDeviceStatus()
    ms_b, ms_p = float(eb.mean()), float(ep.mean())
    return {
        "workload": f"{len(pop)} meshes, CVs log-uniform [500, {cv_max}], 70% "
                    "Catmull-Clark / 30% Loop tori and cubes, uniform L1-4, 3-12 primvars",
        "meshes": len(pop), "stencils_per_frame": n_st, "nnz": nnz,
        "generation_s": gen_s, "generation_factory_s": factory_s,
        "generation": "host topology + masks on all host threads, tables merged on the "
                      "device by GB300StencilTableFactory", "tuned": cfg,
        "batched": {"frame_ms": float(fb.mean()), "eval_ms": ms_b,
                    "stencils_per_s": n_st / (ms_b / 1e3),
                    "frame_ms_p50": float(np.percentile(fb, 50)),
                    "frame_ms_p99": float(np.percentile(fb, 99)),
                    "launches_per_frame": 1},
        "plain_per_mesh": {"frame_ms": float(fp.mean()), "eval_ms": ms_p,
                           "stencils_per_s": n_st / (ms_p / 1e3),
                           "frame_ms_p50": float(np.percentile(fp, 50)),
                           "frame_ms_p99": float(np.percentile(fp, 99)),
                           "launches_per_frame": len(pop)},
        # medians: the plain path enqueues 256 calls from the host, so a host-side stall shows
        # up as an idle gap in its frame, which the mean carries and the median does not
        "speedup_eval": float(np.median(ep) / np.median(eb)),
        "speedup_frame": float(np.median(fp) / np.median(fb)),
        "speedup_eval_mean": ms_p / ms_b,
        "bit_identical_to_plain": identical, "device_status": status,
        "roofline": {"bound": "hbm", "kernel": "k_stencils_batch (persistent, graph replay)",
                     "algorithmic_bytes": b_alg, "achieved": b_alg / (ms_b / 1e3) / 1e9,
                     "peak": peak, "unit": "GB/s", "frac": b_alg / (ms_b / 1e3) / 1e9 / peak,
                     "plain_frac": b_alg / (ms_p / 1e3) / 1e9 / peak},
    }


def bench_serving(args):
    """Serving: a pool of resident topologies under a device-memory budget (LRU), an open-loop
    Poisson request stream with Zipf(1.1) topology popularity, half refine requests (uniform
    level 1-4 of the topology) and half limit requests (10k-1M uniform (face, u, v) points,
    P + dPdu + dPdv); latency = submit -> results in pinned host memory.  The continuous-
    batching server vs the same server serving one request at a time through the plain entry
    points, on the same traces."""
    import torch

    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.server import LIMIT, REFINE, GB300Server

    t0 = time.time()
    pool = workloads.serving_pool(serving_bases(), n_topologies=args.serve_topologies,
                                  cv_max=args.serve_cv_max)
    gen_s = time.time() - t0
    rng = np.random.default_rng(31337)
    # host inputs: per-topology control values, shared query windows, an output ring
    cvs = [torch.from_numpy(workloads.serving_control_values(t, seed=t["id"])).pin_memory()
           for t in pool]
    max_pts = 1_000_000
    uq, vq = (torch.from_numpy(rng.random(max_pts).astype(np.float32)).pin_memory()
              for _ in range(2))
    ut, vt = uq.clone().pin_memory(), vq.clone().pin_memory()
    fold = (ut + vt) > 1.0
    ut[fold], vt[fold] = 1.0 - ut[fold], 1.0 - vt[fold]
    faces = {}
    for t in pool:
        key = (t["scheme"], t["copies"])
        if key not in faces:
            faces[key] = torch.from_numpy(rng.integers(0, t["num_ptex"], max_pts)
                                          .astype(np.int32)).pin_memory()
    ring = torch.empty(args.serve_ring_mb << 18, pin_memory=True)  # floats
    ring_pos = [0]

    def out_slot(n):
        if ring_pos[0] + n > ring.numel():
            ring_pos[0] = 0
        s = ring[ring_pos[0]:ring_pos[0] + n]
        ring_pos[0] += (n + 63) // 64 * 64
        return s

    zipf = 1.0 / np.arange(1, len(pool) + 1) ** 1.1
    zipf /= zipf.sum()
    rank_to_topo = rng.permutation(len(pool))

    def trace(n, rate, seed):
        r = np.random.default_rng(seed)
        arrivals = np.cumsum(r.exponential(1.0 / rate, n))
        arrivals -= arrivals[0]
        topo = rank_to_topo[r.choice(len(pool), n, p=zipf)]
        kinds = np.where(r.random(n) < 0.5, REFINE, LIMIT)
        pts = np.exp(r.uniform(np.log(10_000), np.log(max_pts), n)).astype(np.int64)
        reqs, work = [], 0
        for k in range(n):
            t = pool[topo[k]]
            if kinds[k] == REFINE:
                out = out_slot(len(t["refine"]["sizes"]) * t["length"])
                reqs.append(GB300Server.request(t["id"], REFINE, cvs[t["id"]], out))
                work += len(t["refine"]["sizes"])
            else:
                m = int(pts[k])
                tri = t["base"].triangular
                f = faces[(t["scheme"], t["copies"])][:m]
                u = (ut if tri else uq)[:m]
                v = (vt if tri else vq)[:m]
                reqs.append(GB300Server.request(t["id"], LIMIT, cvs[t["id"]], out_slot(9 * m),
                                                f, u, v))
                work += m
        return reqs, arrivals, work

    def serve(plain):
        srv = GB300Server(int(args.serve_budget_gb * (1 << 30)), 16 << 30,
                          streams=1 if plain else 4, max_requests_per_round=64, plain=plain,
                          pin_host_tables=True)
        for t in pool:
            srv.add_topology(t["id"], t["num_control"], t["length"], t["refine"], t["limit"])
        reqs, arr, _ = trace(args.serve_requests // 2, 5000.0, 7)  # warm-up: hot set resident
        srv.replay(reqs, arr)
        s0 = srv.stats()
        res = []
        for rate in args.serve_rates:
            reqs, arr, work = trace(args.serve_requests, rate, 1000 + int(rate))
            r0 = srv.stats()
            t1 = time.perf_counter()
            lat = srv.replay(reqs, arr)
            wall = time.perf_counter() - t1
            r1 = srv.stats()
            dl = {k: r1[k] - r0[k] for k in r1}
            res.append({"offered_req_per_s": rate, "requests": len(reqs),
                        "achieved_req_per_s": len(reqs) / wall,
                        "evals_per_s": work / wall,
                        "latency_ms": {"p50": float(np.percentile(lat, 50) * 1e3),
                                       "p99": float(np.percentile(lat, 99) * 1e3),
                                       "mean": float(lat.mean() * 1e3)},
                        "time_split": {"wall_s": wall,
                                       "scheduler_launch_s": dl["launchNanos"] / 1e9,
                                       "streams_busy_wait_s": dl["streamsBusyNanos"] / 1e9,
                                       "memory_wait_s": dl["memoryWaitNanos"] / 1e9,
                                       "round_device_s": dl["roundDeviceNanos"] / 1e9,
                                       "rounds": dl["rounds"], "uploads": dl["uploads"],
                                       "upload_gb": dl["bytesUploaded"] / 1e9,
                                       "h2d_gb": dl["h2dBytes"] / 1e9,
                                       "d2h_gb": dl["d2hBytes"] / 1e9}})
        s1 = srv.stats()
        srv.close()
        return res, {k: s1[k] - s0[k] for k in ("rounds", "uploads", "evictions",
                                                 "completed", "failed")} | {
            "host_pinned_gb": s1["hostPinnedBytes"] / 1e9,
            "host_pin_failures": s1["hostPinFailures"],
            "peak_resident_gb": s1["peakResidentBytes"] / 1e9}

    link_before = host_link_gbs()
    batched, bstats = serve(False)
    plain, pstats = serve(True)
    link_after = host_link_gbs()
    table_gb = sum(len(t["refine"]["indices"]) * 8 + len(t["limit"]["pp_indices"]) * 8
                   + len(t["limit"]["patch_indices"]) * 4 for t in pool) / 1e9
    return {
        "workload": f"{len(pool)} topologies (CVs log-uniform [500, {args.serve_cv_max}], "
                    "70% Catmull-Clark / 30% Loop, refine level 1-4, 3-12 primvars), "
                    f"Zipf(1.1) popularity, Poisson arrivals, 50% refine / 50% limit "
                    f"(10k-1M points, P+du+dv), {args.serve_budget_gb} GB table budget",
        "pool_table_gb": table_gb, "generation_s": gen_s,
        "latency_definition": "submit -> results in pinned host memory",
        "host_link_gbs": {"before": link_before, "after": link_after,
                          "note": "pinned 1 GiB copies, median of 5: the serving rounds are "
                                  "bound by this link (results back and table re-uploads)"},
        "batched": {"per_rate": batched, "stats": bstats},
        "plain_one_at_a_time": {"per_rate": plain, "stats": pstats},
    }


METRIC = "stencil evals per s (EvalStencils refine L3 + limit du/dv)"
UNIT = "stencils/s"


def bench_config1(args, stream, peak):
    """The CPU-runnable case: a unit cube with 8 x 8 quads per face (386 control vertices,
    N(0, 0.01) noise), Catmull-Clark uniform level 4 (98,306 stencils of the last level), xyz
    at stride 3, through the device table.  Its 13 MB working set fits in L2, so it is timed
    warm (repeated launches) and cold (a 256 MB buffer written between launches evicts L2),
    median of 50 launches each, CUDA events around the evaluation only.  Beside it: the oracle
    port of CpuEvaluator on one host thread and of OmpEvaluator on all of them (median of 20
    passes after 3 warm-ups) and the error against the oracle."""
    import torch

    from opensubdiv_gb300 import workloads
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilTable)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    w = workloads.refine_cube()
    r = w["refine"]
    n, nnz, ncv = len(r["sizes"]), len(r["indices"]), w["cage"].num_vertices
    t = GB300StencilTable.Create(r["sizes"], r["offsets"], r["indices"], r["weights"])
    src = torch.from_numpy(w["src"]).cuda()
    out = torch.zeros(n * 3, device="cuda")
    d = BD(0, 3, 3)
    flush = torch.empty(64 << 20, device="cuda")

    def one():
        assert Ev.EvalStencilsTable(src, d, out, d, t, stream=stream)

    def timed(cold, reps=50):
        ms = []
        for k in range(reps + 3):
            if cold:
                with torch.cuda.stream(stream):
                    flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one()
            e1.record(stream)
            e1.synchronize()
            if k >= 3:
                ms.append(e0.elapsed_time(e1))
        return float(np.median(ms)), float(np.percentile(ms, 99))

    warm, warm99 = timed(False)
    cold, cold99 = timed(True)
    b = workloads.stencil_bytes(n, nnz, 3, ncv)
    ref = np.zeros(n * 3, np.float32)
    oracle.eval_stencils(w["src"], (0, 3, 3), [ref], [(0, 3, 3)], r["sizes"], r["offsets"],
                         r["indices"], [r["weights"]])
    err = float(np.abs(out.cpu().numpy() - ref).max())
    diag = w["cage"].bbox_diagonal()

    def cpu(threads, reps=20):
        o = np.zeros(n * 3, np.float32)
        ts = []
        for k in range(reps + 3):
            t0 = time.perf_counter()
            oracle.eval_stencils(w["src"], (0, 3, 3), [o], [(0, 3, 3)], r["sizes"], r["offsets"],
                                 r["indices"], [r["weights"]], threads=threads)
            if k >= 3:
                ts.append(time.perf_counter() - t0)
        return n / float(np.median(ts))

    return {"workload": w["name"], "stencils": n, "nnz": nnz, "algorithmic_bytes": b,
            "warm": {"ms": warm, "p99_ms": warm99, "stencils_per_s": n / (warm / 1e3),
                     "achieved_gbs": b / (warm / 1e3) / 1e9},
            "cold_l2": {"ms": cold, "p99_ms": cold99, "stencils_per_s": n / (cold / 1e3),
                        "achieved_gbs": b / (cold / 1e3) / 1e9,
                        "frac_of_hbm_peak": b / (cold / 1e3) / 1e9 / peak,
                        "flush": "256 MB buffer written on the stream before each launch"},
            "accuracy": {"max_abs_err_vs_oracle": err, "bbox_diag": diag,
                         "in_units_of_1e-5_diag": err / (1e-5 * diag)},
            "cpu_port_1_thread_stencils_per_s": cpu(1),
            "cpu_port_all_threads_stencils_per_s": cpu(os.cpu_count() or 1),
            "cpu_threads": os.cpu_count()}


def bench_layouts(w, stream):
    """Device-table EvalStencils on the headline tables per source layout (refine pass, one
    output; limit pass, P+du+dv) and, at 8 floats, per output count 1-6 over a limit table
    carrying 6 weight arrays (du/dv weights reused for the second derivatives: timing only).
    CUDA events on the launch stream, 20 launches after 3 warm-ups, milliseconds."""
    import torch

    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilTable)
    r, lim = w["refine"], w["limit"]
    ncv = w["cage"].num_vertices
    n, m = len(r["sizes"]), len(lim["sizes"])
    t_ref = GB300StencilTable.Create(r["sizes"], r["offsets"], r["indices"], r["weights"])
    ws = [lim["weights"], lim["du_weights"], lim["dv_weights"], lim["du_weights"],
          lim["dv_weights"], lim["du_weights"]]
    t6 = GB300StencilTable.Create(lim["sizes"], lim["offsets"], lim["indices"], *ws)

    def timeit(fn, k=20):
        for _ in range(3):
            assert fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            assert fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return round(e0.elapsed_time(e1) / k, 4)

    keys = ("du", "dv", "duu", "duv", "dvv")
    res = {"refine_ms": {}, "limit_P_du_dv_ms": {}, "limit_L8_ms_by_outputs": {}}
    for ln, st in ((3, 4), (4, 4), (8, 8), (12, 12)):
        src = torch.rand(ncv * st, device="cuda")
        o = [torch.zeros(max(n, m) * ln, device="cuda") for _ in range(6)]
        sd, dd = BD(0, ln, st), BD(0, ln, ln)
        res["refine_ms"][f"L{ln}/stride{st}"] = timeit(
            lambda: Ev.EvalStencilsTable(src, sd, o[0], dd, t_ref, stream=stream))
        res["limit_P_du_dv_ms"][f"L{ln}/stride{st}"] = timeit(
            lambda: Ev.EvalStencilsTable(src, sd, o[0], dd, t6, du=o[1], duDesc=dd, dv=o[2],
                                         dvDesc=dd, stream=stream))
        if ln == 8:
            for nout in range(1, 7):
                kw = {}
                for k in range(1, nout):
                    kw[keys[k - 1]], kw[keys[k - 1] + "Desc"] = o[k], dd
                res["limit_L8_ms_by_outputs"][str(nout)] = timeit(
                    lambda: Ev.EvalStencilsTable(src, sd, o[0], dd, t6, stream=stream, **kw))
    res["stencils"] = {"refine": n, "limit": m}
    return res


def bench_factory(args, w):
    """Stencil-table construction for the refine workload's cage (the step before the path):
    the GPU factory (host topology + Far-form masks, then GB300StencilTableFactory: mask upload
    and device merge, table left on the device) against the host generator (topology + OpenMP
    composition in double + upload of the finished table), plus the oracle's restatement of
    Far's single-threaded StencilBuilder merge on a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from opensubdiv_gb300 import shapes, topology
    from opensubdiv_gb300.evaluator import GB300StencilTable, GB300StencilTableFactory as F

    cage, level = w["cage"], w["level"]
    reps = 3
    t0 = time.perf_counter()
    topo = topology.UniformRefiner(cage, level, stencils=False)
    t_topo = time.perf_counter() - t0
    t0 = time.perf_counter()
    nc, levels = topo.factory_masks()
    t_masks = time.perf_counter() - t0
    mask_nnz = sum(len(d["sources"]) for d in levels)
    F.Create(nc, levels, generateIntermediateLevels=False)  # warm-up (module, pools)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        tab = F.Create(nc, levels, generateIntermediateLevels=False)
        times.append(time.perf_counter() - t0)
        del tab
    t_gpu = float(np.median(times))
    launches0 = _lib_launches()
    tab = F.Create(nc, levels, generateIntermediateLevels=False)
    launches = _lib_launches() - launches0
    n, nnz = tab.GetNumStencils(), tab.GetNumIndices()
    # host generator path for the same table (its tables are what the refine bench uses)
    r = w["refine"]
    t0 = time.perf_counter()
    gen = topology.UniformRefiner(cage, level)
    g = gen.stencil_table()
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    up = GB300StencilTable.Create(g["sizes"], g["offsets"], g["indices"], g["weights"])
    t_up = time.perf_counter() - t0
    # same stencils: sizes identical, weights within 2 float ulps of 1 (float vs double sums)
    a, b = tab.CopyToHost(), up.CopyToHost()
    same = bool(np.array_equal(a["sizes"], b["sizes"]) and np.array_equal(a["indices"],
                                                                        b["indices"]))
    werr = float(np.abs(a["weights"] - b["weights"]).max()) if same else None
    del up, gen, g
    # Far's merge restated (oracle, one thread) on a bounded sample: a smaller torus
    sn, sv = max(8, args.nu // 4), max(8, args.nv // 4)
    scage = shapes.torus(sn, sv, tri_fraction=0.05, crease_fraction=0.02, seed=2024)
    snc, slev = topology.UniformRefiner(scage, level, stencils=False).factory_masks()
    t0 = time.perf_counter()
    st = oracle.factory_create(snc, slev, intermediate=False)
    t_orc = time.perf_counter() - t0
    return {
        "workload": f"{w['name'].split('_')[0]} Catmark L{level}: {n} stencils, {nnz} entries "
                    f"from {mask_nnz} mask entries",
        "stencils": n, "entries": int(nnz), "mask_entries": int(mask_nnz),
        "host_topology_ms": t_topo * 1e3, "host_masks_ms": t_masks * 1e3,
        "gpu_factory_ms": t_gpu * 1e3, "gpu_factory_launches": int(launches),
        "gpu_path_ms": (t_topo + t_masks + t_gpu) * 1e3,
        "host_generator_ms": t_gen * 1e3, "host_upload_ms": t_up * 1e3,
        "host_path_ms": (t_gen + t_up) * 1e3,
        "speedup_path": (t_gen + t_up) / (t_topo + t_masks + t_gpu),
        "gpu_factory_stencils_per_s": n / t_gpu,
        "matches_host_generator": same, "max_weight_diff": werr,
        "far_merge_port": {"stencils_per_s": len(st["sizes"]) / t_orc, "cores": 1,
                           "sample": f"torus {sn}x{sv} L{level} ({len(st['sizes'])} stencils, "
                                     "oracle restatement of StencilBuilder's merge)"},
    }


def _lib_launches():
    from opensubdiv_gb300 import _lib
    return int(_lib.load().GB300GetLaunchCount())


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_key):
    """Per-launch DRAM bytes of the kernel from the committed ncu summary, if any."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for f in sorted(os.listdir(d)):
        if not f.endswith(".md"):
            continue
        for line in open(os.path.join(d, f)):
            m = re.match(r"\s*dram_bytes_per_launch\[(\S+)\]:\s*([0-9.eE+]+)", line)
            if m and m.group(1) == kernel_key:
                return float(m.group(2))
    return None


class NvmlClocks:
    """Read-only NVML polling (SM clock, max clock, clock-event reasons) every 2 ms in a
    thread, so even a short timed region gets samples.  Reasons bits per nvml.h:
    0x4 sw_power_cap, 0x8 hw_slowdown, 0x20 sw_thermal_slowdown, 0x40 hw_thermal_slowdown."""

    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
            0x40: "hw_thermal_slowdown"}

    def __init__(self, index=0):
        import ctypes

        self.C = ctypes
        self.nv = ctypes.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        if self.nv.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        self.sm, self.reasons, self.stop = [], 0, False
        mx = ctypes.c_uint()
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx))
        self.max = float(mx.value)

    def _loop(self):
        C = self.C
        mhz, r = C.c_uint(), C.c_ulonglong()
        get_r = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop:
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0:
                self.sm.append(float(mhz.value))
            if get_r(self.h, C.byref(r)) == 0:
                self.reasons |= int(r.value)
            time.sleep(0.002)

    def __enter__(self):
        self.t = threading.Thread(target=self._loop, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop = True
        self.t.join(timeout=2)

    def summary(self):
        return {"sm_mhz": float(np.median(self.sm)) if self.sm else None, "sm_max_mhz": self.max,
                "reasons": sorted(n for b, n in self.BITS.items() if self.reasons & b),
                "samples": len(self.sm), "source": "nvml"}


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region (fallback when NVML
    cannot be loaded)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 8:
                continue
            for k, n in enumerate(names):
                if r[4 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_passes(w, reps, warmup, threads, fraction=1.0):
    """Seconds of each of `reps` timed passes (after `warmup` untimed ones) of the oracle port
    of CpuEvaluator / OmpEvaluator (OpenMP over `threads`) over the first `fraction` of the
    refine and limit tables, and the stencils one pass evaluates."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    L = w["length"]
    r, l = w["refine"], w["limit"]
    n_r, n_l = int(len(r["sizes"]) * fraction), int(len(l["sizes"]) * fraction)
    out = np.zeros(len(r["sizes"]) * L, np.float32)
    outs = [np.zeros(len(l["sizes"]) * L, np.float32) for _ in range(3)]
    d = (0, L, L)

    def one():
        oracle.eval_stencils(w["src"], d, [out], [d], r["sizes"], r["offsets"], r["indices"],
                             [r["weights"]], 0, n_r, threads=threads)
        oracle.eval_stencils(w["src"], d, outs, [d] * 3, l["sizes"], l["offsets"], l["indices"],
                             [l["weights"], l["du_weights"], l["dv_weights"]], 0, n_l,
                             threads=threads)

    for _ in range(warmup):
        one()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        one()
        times.append(time.perf_counter() - t0)
    return times, n_r + n_l


def host_cpu():
    """nproc and the CPU model of this host (lscpu, else /proc/cpuinfo)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model and os.path.exists("/proc/cpuinfo"):
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                model = line.split(":", 1)[1].strip()
                break
    return {"nproc": os.cpu_count(), "cpu_model": model}


def cpu_baseline(w, reps=20, warmup=3, single_fraction=1.0 / 16):
    """CPU baseline on this host: the median of `reps` timed passes after `warmup` untimed
    ones, over all host threads (the OmpEvaluator form) and on one thread (the CpuEvaluator
    form, over the first `single_fraction` of the tables per pass)."""
    threads = os.cpu_count() or 1
    t_all, n_all = cpu_passes(w, reps, warmup, threads)
    t_one, n_one = cpu_passes(w, reps, warmup, 1, single_fraction)
    med_all, med_one = float(np.median(t_all)), float(np.median(t_one))
    return {"value": n_all / med_all, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"median of {reps} full refine + limit passes after {warmup} warm-ups "
                      "(oracle port of OmpEvaluator: OpenMP over all host threads)",
            "pass_ms": {"median": 1e3 * med_all, "p99": 1e3 * float(np.percentile(t_all, 99))},
            "single_thread": {
                "value": n_one / med_one, "unit": UNIT, "cores": 1,
                "sample": f"median of {reps} passes over the first {single_fraction:.4g} of the "
                          f"refine and limit tables ({n_one} stencils) after {warmup} warm-ups "
                          "(oracle port of CpuEvaluator, one thread)",
                "pass_ms": {"median": 1e3 * med_one,
                            "p99": 1e3 * float(np.percentile(t_one, 99))}},
            "host": host_cpu()}


def reference_cuda(args, w):
    """The reference's own CUDA evaluator kernels (osd/cudaKernel.cu built for sm_103a into
    oracle/_ref by the oracle recipe) with its own launch logic, on the same workloads: refine
    EvalStencils, limit EvalStencils with du/dv (one CudaEvalStencils per weight array, as
    CudaEvaluator does), and EvalPatches with all derivatives at the bench's query points (patch
    coords from the oracle's PatchMap on the host).  CUDA events per launch group."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import refcuda
        import torch
    except ImportError as e:
        return {"unavailable": str(e)}
    if not refcuda.available():
        return {"unavailable": "oracle/_ref/osd_cudaKernel.cubin not built (reference sources "
                               "absent where build() ran)"}
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    import oracle
    from opensubdiv_gb300 import workloads
    L = w["length"]
    r, lim = w["refine"], w["limit"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    src = dev(w["src"])
    rt = [dev(r[k]) for k in ("sizes", "offsets", "indices", "weights")]
    lt = [dev(lim[k]) for k in ("sizes", "offsets", "indices")]
    lw = [dev(lim[k]) for k in ("weights", "du_weights", "dv_weights")]
    n_ref, n_lim = len(r["sizes"]), len(lim["sizes"])
    out = torch.empty(n_ref * L, device="cuda")
    lo = [torch.empty(n_lim * L, device="cuda") for _ in range(3)]

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    refine_ms = timed(lambda: refcuda.eval_stencils(
        src.data_ptr(), out.data_ptr(), L, L, L, *[t.data_ptr() for t in rt], 0, n_ref))
    limit_ms = timed(lambda: refcuda.eval_stencils_derivatives(
        src.data_ptr(), [o.data_ptr() for o in lo], L, L, [L] * 3, *[t.data_ptr() for t in lt],
        [x.data_ptr() for x in lw], 0, n_lim))
    res = {"kernels": "osd/cudaKernel.cu (computeStencils<<<512,32>>> for L=8; "
                      "computePatches<<<512,32>>>)",
           "refine_ms": refine_ms, "limit_ms": limit_ms,
           "stencils_per_s": (n_ref + n_lim) / ((refine_ms + limit_ms) / 1e3)}
    # the CPU-runnable cube (xyz, stride 3: computeStencilsNv<3>), warm
    cw = workloads.refine_cube()
    cr = cw["refine"]
    csrc = dev(cw["src"])
    ct = [dev(cr[k]) for k in ("sizes", "offsets", "indices", "weights")]
    cout = torch.empty(len(cr["sizes"]) * 3, device="cuda")
    c_ms = timed(lambda: refcuda.eval_stencils(
        csrc.data_ptr(), cout.data_ptr(), 3, 3, 3, *[x.data_ptr() for x in ct], 0,
        len(cr["sizes"])))
    res["config1_cube"] = {"workload": cw["name"], "refine_ms_warm": c_ms,
                           "stencils_per_s": len(cr["sizes"]) / (c_ms / 1e3)}
    if not args.no_patches:
        from opensubdiv_gb300 import workloads
        pw = patch_workload(args.patch_points)
        handles = oracle.PatchMap(pw["arrays"], pw["params"], pw["triangular"]).find(
            pw["face"], pw["u"], pw["v"])
        coords = dev(oracle.make_coords(handles, pw["u"], pw["v"]))
        n = len(pw["face"])
        psrc = dev(pw["src"])
        pa, pi, pp = dev(pw["arrays"]), dev(pw["indices"]), dev(pw["params"])
        outs = [torch.empty(n * 3, device="cuda") for _ in range(6)]
        patches_ms = timed(lambda: refcuda.eval_patches(
            psrc.data_ptr(), [o.data_ptr() for o in outs], 3, 3, [3] * 6, n, coords.data_ptr(),
            pa.data_ptr(), pi.data_ptr(), pp.data_ptr()))
        res.update(eval_patches_ms=patches_ms, patch_points=n,
                   patch_evals_per_s=n / (patches_ms / 1e3))
    return res


def run_reference(args, rank, world):
    if rank != 0:
        return
    # the workload generator built by the oracle recipe: this process maps no library of
    # the package (oracle/_build and oracle/_ref only)
    from opensubdiv_gb300 import topology, workloads
    gen = os.path.join(ROOT, "oracle", "_build", "libworkload_topology.so")
    if not os.path.exists(gen):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "workload"],
                       check=True)
    topology.use_library(gen)

    w = workloads.refine_and_limit_torus(args.nu, args.nv, n_limit=args.n_limit)
    threads = os.cpu_count() or 1
    # one step = one full refine + limit pass over all host threads; value = the median
    times, n_step = cpu_passes(w, args.steps, args.warmup, threads)
    med = float(np.median(times))
    value = n_step / med
    base = cpu_baseline(w, reps=max(args.steps, 20), warmup=max(args.warmup, 3))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * med, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded torus cage)",
            "config": {"workload": w["name"], "stencils_per_step": n_step,
                       "refine_stencils": len(w["refine"]["sizes"]),
                       "refine_nnz": int(len(w["refine"]["indices"])),
                       "limit_stencils": len(w["limit"]["sizes"]),
                       "limit_nnz": int(len(w["limit"]["indices"])), "primvars": w["length"],
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"median of {args.steps} full refine + limit passes "
                                       f"after {args.warmup} warm-ups (oracle port of "
                                       "OmpEvaluator: OpenMP over all host threads)",
                             "single_thread": base["single_thread"], "host": base["host"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "reference_cuda": reference_cuda(args, w)}
    print(json.dumps(line), flush=True)


def run_gb300(args, rank, world):
    import torch

    from opensubdiv_gb300 import _lib, workloads
    from opensubdiv_gb300.evaluator import (BufferDescriptor as BD, GB300Evaluator as Ev,
                                            GB300StencilTable, GB300VertexBuffer)

    from opensubdiv_gb300 import replicas

    local = replicas.world()[1]
    torch.cuda.set_device(local)
    _lib.load()
    dist = replicas.init("nccl")

    w = workloads.refine_and_limit_torus(args.nu, args.nv, n_limit=args.n_limit)
    L = w["length"]
    r, lim = w["refine"], w["limit"]
    ncv = w["cage"].num_vertices
    n_ref, n_lim = len(r["sizes"]), len(lim["sizes"])
    stream = torch.cuda.Stream()
    t_ref = GB300StencilTable.Create(r["sizes"], r["offsets"], r["indices"], r["weights"])
    t_lim = GB300StencilTable.Create(lim["sizes"], lim["offsets"], lim["indices"],
                                     lim["weights"], lim["du_weights"], lim["dv_weights"])
    vb = GB300VertexBuffer.Create(L, ncv)
    vb.UpdateData(w["src"], 0, ncv)
    src = vb.BindCudaBuffer()
    out = torch.empty(n_ref * L, device="cuda")
    lo = [torch.empty(n_lim * L, device="cuda") for _ in range(3)]
    d = BD(0, L, L)

    def step():
        ok1 = Ev.EvalStencilsTable(src, d, out, d, t_ref, stream=stream)
        ok2 = Ev.EvalStencilsTable(src, d, lo[0], d, t_lim, du=lo[1], duDesc=d, dv=lo[2],
                                   dvDesc=d, stream=stream)
        assert ok1 and ok2, _lib.last_error()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    # ---- device-resident timing (value) + per-launch events for the roofline ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = _lib.launch_count()
    try:
        sampler = NvmlClocks(local)
    except OSError:
        sampler = ClockSampler(local)
    with sampler as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            t_start.record(stream)
            for k in range(args.steps):
                ev[k][0].record(stream)
                assert Ev.EvalStencilsTable(src, d, out, d, t_ref, stream=stream)
                ev[k][1].record(stream)
                assert Ev.EvalStencilsTable(src, d, lo[0], d, t_lim, du=lo[1], duDesc=d,
                                            dv=lo[2], dvDesc=d, stream=stream)
                ev[k][2].record(stream)
            t_end.record(stream)
        barrier()
    launches = _lib.launch_count() - launches0
    ms = t_start.elapsed_time(t_end)
    ref_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in ev]))
    lim_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in ev]))
    ms = replicas.max_over_ranks(dist, ms, device="cuda")
    n_step = n_ref + n_lim
    value = replicas.job_rate(n_step * args.steps, world, ms / 1e3)

    # ---- end to end through the C ABI with host buffers ----
    host_src = torch.from_numpy(w["src"].copy()).pin_memory()
    host_out = torch.empty(n_ref * L, pin_memory=True)
    host_lo = [torch.empty(n_lim * L, pin_memory=True) for _ in range(3)]
    phase = np.random.default_rng(7).uniform(0, 2 * np.pi)
    base = w["src"].reshape(ncv, L)

    # Steps are pipelined: step k evaluates into output set k % 2 on `stream` while a copy
    # stream reads step k - 1's outputs back, so the host-link transfer (the bound) overlaps
    # evaluation.  Every step still copies its inputs in and all of its outputs out.
    copy_stream = torch.cuda.Stream()
    outs2 = [(out, lo), (torch.empty_like(out), [torch.empty_like(x) for x in lo])]
    evaluated = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]

    def e2e_step(k):
        o, l = outs2[k % 2]
        vb.UpdateData(host_src.numpy(), 0, ncv, stream=stream)  # pinned -> HBM
        stream.wait_event(copied[k % 2])  # the copy of step k - 2 has read this set
        assert Ev.EvalStencilsTable(src, d, o, d, t_ref, stream=stream)
        assert Ev.EvalStencilsTable(src, d, l[0], d, t_lim, du=l[1], duDesc=d, dv=l[2],
                                    dvDesc=d, stream=stream)
        evaluated[k % 2].record(stream)
        copy_stream.wait_event(evaluated[k % 2])
        with torch.cuda.stream(copy_stream):
            host_out.copy_(o, non_blocking=True)
            for a, b in zip(host_lo, l):
                a.copy_(b, non_blocking=True)
        copied[k % 2].record(copy_stream)

    # per-frame deformation of the control points (host side, outside the copy/eval timing)
    host_src.numpy().reshape(ncv, L)[:, :3] = base[:, :3] * (1.0 + 0.01 * np.sin(phase))
    for k in range(args.warmup):
        e2e_step(k)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        e2e_step(k)
    stream.wait_stream(copy_stream)  # the last step's outputs are on the host
    e1.record(stream)
    barrier()
    e2e_ms = e0.elapsed_time(e1)
    e2e_ms = replicas.max_over_ranks(dist, e2e_ms, device="cuda")
    e2e_value = replicas.job_rate(n_step * args.steps, world, e2e_ms / 1e3)
    h2d = ncv * L * 4
    d2h = (n_ref + 3 * n_lim) * L * 4

    # correctness spot check against the oracle on a slice (cheap, outside timing)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    k0, k1 = n_ref // 2, n_ref // 2 + 20000
    refv = np.zeros(n_ref * L, np.float32)
    oracle.eval_stencils(host_src.numpy(), (0, L, L), [refv], [(0, L, L)], r["sizes"],
                         r["offsets"], r["indices"], [r["weights"]], k0, k1, threads=4)
    spot = float(np.abs(host_out.numpy()[k0 * L:k1 * L] - refv[k0 * L:k1 * L]).max())
    diag = w["cage"].bbox_diagonal()

    if rank != 0:
        return
    peak, peak_kind = peaks()
    b_ref = workloads.stencil_bytes(n_ref, len(r["indices"]), L, ncv)
    b_lim = workloads.stencil_bytes(n_lim, len(lim["indices"]), L, ncv, n_weight_arrays=3,
                                    n_outputs=3)
    achieved = b_ref / (ref_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded torus cage, stencils from the native uniform refiner)",
        "config": {"workload": w["name"], "stencils_per_step": n_step, "refine_stencils": n_ref,
                   "refine_nnz": int(len(r["indices"])), "limit_stencils": n_lim,
                   "limit_nnz": int(len(lim["indices"])), "primvars": L,
                   "l2": "per-step working set 1.4 GB > 129 MB L2 (no flush needed)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": "k_stencils_sell<1,8> (refine EvalStencils, sliced layout, staged ring)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": b_ref, "launch_ms": ref_ms,
                     "traffic": ncu_traffic("refine"),
                     "limit_kernel": {"launch_ms": lim_ms, "algorithmic_bytes": b_lim,
                                      "achieved": b_lim / (lim_ms / 1e3) / 1e9}},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms / args.steps,
                "pipelining": "step k evaluates while step k-1's outputs are read back "
                              "(two output sets); every step copies all inputs and outputs"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "accuracy": {"max_abs_err_vs_oracle_slice": spot, "bbox_diag": diag,
                     "rel": spot / diag},
    }
    if not args.no_config1:
        line["config1_cube"] = bench_config1(args, stream, peak)
    if not args.no_patches:
        line["eval_patches"] = bench_patches(args, stream, peak)
        line["eval_patches_loop"] = bench_patches(args, stream, peak, loop=True)
    if not args.no_bfr:
        line["bfr_tessellation"] = bench_bfr(args, stream, peak)
    # serving first: its host-link-bound rounds measure lower after the batching section's
    # 200 GB of tables have churned device and host memory
    if not args.no_serving:
        release_memory()
        line["serving"] = bench_serving(args)
    if not args.no_batch:
        release_memory()
        line["batching"] = bench_batch(args, stream, peak, args.batch_cv_max)
        release_memory()
        if args.batch_cv_max_scaled > 0:
            line["batching_scaled"] = bench_batch(args, stream, peak, args.batch_cv_max_scaled)
            release_memory()
    if not args.no_factory:
        line["factory"] = bench_factory(args, w)
    if args.layouts:
        line["layouts"] = bench_layouts(w, stream)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    from opensubdiv_gb300 import replicas
    rank, _, world = replicas.world()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gb300(args, rank, world)


if __name__ == "__main__":
    main()
