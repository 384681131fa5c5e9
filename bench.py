#!/usr/bin/env python
"""Headline benchmark: cone-beam CGLS iterations/s on one GB300.

Workload (default ``cone512``): 512^3 ellipsoid phantom, 720 views over 2*pi,
1024x768 flat panel at 0.5 mm, source-isocentre 600 mm, source-detector
1200 mm, 0.5 mm voxels. A step is one CGLS iteration on (A^T A + lam I) u = b,
b = A^T A x_true, with the matched Siddon projector pair:

* ``value``: the graph form (FP32 storage, fused updates with FP64 reductions
  and device-side alpha/beta, one iteration replayed as a CUDA graph), inputs
  resident in HBM;
* ``detail.mixed_iter_per_s``: the same with an FP16 copy of the projected
  direction (FP32 accumulation, FP32 residual refresh every 10 iterations);
* ``detail.plain_iter_per_s``: plain FP32, one kernel per vector operation,
  scalars synchronised to the host every iteration;
* ``e2e``: the graph form through the host-buffer C-ABI call
  (fl_cgls_solve_host: b and u0 copied in, u copied out, inside the timing);
* ``roofline``: the dominant projector kernel, algorithmic bytes
  (sum over rays of voxels crossed x voxel bytes + rays x sinogram bytes,
  crossings counted on the GPU) over its CUDA-event time;
* ``cpu_baseline``: the reference's CPU projector pair (the oracle's bit-exact
  restatement) timed on a bounded sample on this host and extrapolated.

``--impl reference`` times that CPU path alone as the reference arm.
Multi-GPU: replicas only (independent solves per rank, no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # 512^3 cone CGLS with gradients (the large cone-beam configuration)
    "cone512": dict(n=512, nv=720, na=1024, nb=768, det_mm=0.5, SO=600.0, SD=1200.0,
                    vox_mm=0.5, lam=0.0),
    # 256^3 circular cone projector pair
    "cone256": dict(n=256, nv=360, na=512, nb=384, det_mm=1.0, SO=600.0, SD=1200.0,
                    vox_mm=1.0, lam=0.0),
    # small case for ncu captures
    "cone128": dict(n=128, nv=90, na=256, nb=192, det_mm=2.0, SO=600.0, SD=1200.0,
                    vox_mm=2.0, lam=0.0),
}
REFRESH = 10


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cone512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--only", default="", help="comma list of legs: mixed,plain,e2e,kernels")
    return ap.parse_args()


def para_of(w):
    from framelab_gb300 import geometry as G
    return G.cone_para_mm(w["n"], w["nv"], w["na"], w["nb"], det_pitch_mm=w["det_mm"],
                          SO_mm=w["SO"], SD_mm=w["SD"], voxel_mm=w["vox_mm"])


# --------------------------------------------------------------------------
# CPU leg: the reference's CPU projector pair (oracle restatement, bit-exact)
# --------------------------------------------------------------------------
def cpu_sample(w, p):
    """Times Ax_cone_mf_cpu_siddon and Atx_cone_mf_cpu_new (the oracle's bit-exact
    restatement of the reference's CPU kernels) on a bounded sample with all host
    threads and extrapolates one CGLS iteration (one forward projection + one
    backprojection; the vector algebra is negligible next to them).
    Forward sample: one view per thread, every 16th detector row (a ray depends
    only on its view, column and row, so these are rays of the full scan).
    Backprojection sample: one slice per thread, spread over z, x 4 views."""
    import oracle as O
    threads = max(1, os.cpu_count() or 1)
    n, nv, nb = w["n"], w["nv"], w["nb"]
    rng = np.random.default_rng(0)
    x = rng.random(n ** 3, dtype=np.float32)
    fv = min(nv, threads)
    rows = np.arange(0, nb, 16)
    q = dict(p)
    q["sd_phi"] = p["sd_phi"][:fv]
    q["sd_z"] = p["sd_z"][:fv]
    q["z_det"] = p["z_det"][rows]
    q["id_X"] = p["id_X"][:fv]
    t0 = time.perf_counter()
    O.cone_siddon_f32(x, q, threads=threads)
    t_f = time.perf_counter() - t0
    fwd_full = t_f * (nv / fv) * (nb / len(rows))
    av = 4
    y = rng.random(av * w["na"] * nb, dtype=np.float32)
    r = dict(p)
    for k in ("cos_phi", "sin_phi", "sd_phi", "sd_z"):
        r[k] = p[k][:av]
    r["id_Y"] = np.arange(av, dtype=np.uint32).reshape(av, 1)
    r["Nv"] = np.array([av], np.uint32)
    r["tmp_size"] = np.uint32(av)
    zs = min(threads, n)
    zsel = np.linspace(0, n - 1, zs).astype(int)
    t0 = time.perf_counter()
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda z: O.cone_adj_f32(y, r, threads=1, slices=(int(z), int(z) + 1)), zsel))
    t_a = time.perf_counter() - t0
    adj_full = t_a * (n / zs) * (nv / av)
    it_s = fwd_full + adj_full
    return dict(value=1.0 / it_s, unit="iter/s", cores=threads, kind="port",
                sample=(f"Ax_cone_mf_cpu_siddon on {fv}/{nv} views x {len(rows)}/{nb} rows "
                        f"({t_f:.2f} s) + Atx_cone_mf_cpu_new on {zs}/{n} slices x {av}/{nv} "
                        f"views ({t_a:.2f} s), {threads} threads, extrapolated linearly to one "
                        f"forward + backprojection ({it_s:.0f} s per CGLS iteration)"))


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.rows.append([c.strip() for c in ln.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if len(r) > 3 + k and r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


# --------------------------------------------------------------------------
def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[a.workload]
    config = {"workload": f"{a.workload}: {w['n']}^3 cone CGLS, {w['nv']} views, "
                          f"{w['na']}x{w['nb']} panel @ {w['det_mm']} mm, SO {w['SO']:.0f} mm, "
                          f"SD {w['SD']:.0f} mm, voxel {w['vox_mm']} mm",
              "global_batch": world, "l2": "working set > L2 (volume and sinogram >= 64 MiB "
                                            "per operand; 512^3: 0.5 GiB + 2.2 GiB)",
              "parallelism": f"replicas{world}"}
    metric = "CGLS iter/s (cone-beam, matched Siddon pair, fused FP32 graph form)"

    if a.impl == "reference":
        if rank != 0:
            return
        p = para_of(w)
        for _ in range(a.warmup):
            cpu_sample(w, p)
        t0 = time.perf_counter()
        samples = [cpu_sample(w, p) for _ in range(a.steps)]
        el = time.perf_counter() - t0
        v = float(np.median([s_["value"] for s_ in samples])) if samples else None
        out = {"metric": metric, "value": v, "unit": "iter/s", "n_gpus": 0, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": 1000.0 / v if v else None,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": "synthetic (seeded random volume and sinogram)",
               "impl": "reference", "config": config,
               "cpu_baseline": {"value": v, "unit": "iter/s", "cores": samples[0]["cores"] if samples else None,
                                "kind": "port", "sample": samples[0]["sample"] if samples else ""},
               "e2e": {"value": v, "unit": "iter/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0},
               "wall_s": el}
        print(json.dumps(out))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from framelab_gb300 import phantoms as PH
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def tmax(t):
        if world > 1:
            import torch.distributed as dist
            x = torch.tensor([t], device=dev, dtype=torch.float64)
            dist.all_reduce(x, op=dist.ReduceOp.MAX)
            return float(x.item())
        return t

    legs = set(a.only.split(",")) if a.only else {"mixed", "plain", "e2e", "kernels"}
    legs.add("graph")
    p = para_of(w)
    P = Plan(p)
    n = w["n"]
    x_true = torch.from_numpy(PH.ellipsoids_3d(n, seed=5).reshape(-1)).to(dev)
    f = P.forward(x_true)
    b = P.adjoint(f).reshape(-1)
    del f
    torch.cuda.synchronize()
    lam = w["lam"]
    K, W = a.steps, a.warmup
    stream = torch.cuda.current_stream()
    detail = {}

    def timed(fn):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return out, tmax(e0.elapsed_time(e1) / 1000.0)

    # ---- graph form (headline) ----
    cg_g = NativeCGLS(P, "graph")
    if W:
        cg_g.solve(b, lam=lam, iters=W)
    clocks = ClockSampler(local)
    with clocks:
        u_g, t_g = timed(lambda: cg_g.solve(b, lam=lam, iters=K))
    value = world * K / t_g
    detail["graph_iter_per_s_per_gpu"] = K / t_g
    xt = x_true.double()

    def rel(a_, b_):
        return (torch.linalg.vector_norm((a_ - b_).double()) /
                torch.linalg.vector_norm(b_.double())).item()

    detail["graph_vs_truth_rel_l2"] = rel(u_g, xt)

    # ---- mixed (FP16 direction) and plain FP32 forms ----
    if "mixed" in legs:
        cg_m = NativeCGLS(P, "mixed")
        if W:
            cg_m.solve(b, lam=lam, iters=W, refresh=REFRESH)
        u_m, t_m = timed(lambda: cg_m.solve(b, lam=lam, iters=K, refresh=REFRESH))
        detail["mixed_iter_per_s"] = world * K / t_m
        detail["mixed_vs_graph_rel_l2"] = rel(u_m, u_g)
        del cg_m, u_m
    if "plain" in legs:
        cg_p = NativeCGLS(P, "plain")
        if W:
            cg_p.solve(b, lam=lam, iters=W)
        u_p, t_p = timed(lambda: cg_p.solve(b, lam=lam, iters=K))
        detail["plain_iter_per_s"] = world * K / t_p
        detail["graph_over_plain"] = t_p / t_g
        detail["mixed_over_plain"] = (detail["mixed_iter_per_s"] / detail["plain_iter_per_s"]
                                      if "mixed_iter_per_s" in detail else None)
        detail["graph_vs_plain_rel_l2"] = rel(u_g, u_p)
        del cg_p, u_p

    # ---- e2e: host buffers through the C ABI ----
    e2e = None
    if "e2e" in legs:
        bh = torch.empty(b.numel(), dtype=torch.float32, pin_memory=True)
        bh.copy_(b.cpu())
        uh = torch.zeros(b.numel(), dtype=torch.float32, pin_memory=True)
        bn, un = bh.numpy(), uh.numpy()
        cg_g.solve_host(bn, un, lam=lam, iters=max(W, 1))
        _, t_e = timed(lambda: cg_g.solve_host(bn, un, lam=lam, iters=K))
        nb = b.numel() * 4
        e2e = {"value": world * K / t_e, "unit": "iter/s",
               "h2d_bytes_per_step": nb / K, "d2h_bytes_per_step": nb / K,
               "call": f"fl_cgls_solve_host, {K} iterations per call: b in, u out "
                       "(u0 = 0 needs no copy)"}

    # ---- projector kernels: algorithmic bytes and CUDA-event times ----
    roofline = None
    launches = 5 * K + 1          # graph form: fwd, adj, 3 fused updates per iteration + init
    if "kernels" in legs:
        from framelab_gb300 import _lib
        L = _lib.load()
        cnt = P.count_intersections()
        n_isect = int(cnt.sum(dtype=torch.int64).item())
        del cnt
        n_rays = P.n_rays
        p32 = (u_g / (u_g.abs().max() + 1e-30)).contiguous()
        ysc = torch.empty(n_rays, device=dev, dtype=torch.float32)
        xo = torch.empty(P.n_vox, device=dev, dtype=torch.float32)
        import ctypes as C
        from framelab_gb300.projector import DTYPES
        reps = 3

        def run_fwd():
            for _ in range(reps):
                _lib.check(L.fl_forward(P.handle, 16, p32.data_ptr(), DTYPES[torch.float32],
                                        ysc.data_ptr(), DTYPES[torch.float32], stream.cuda_stream))

        def run_adj():
            for _ in range(reps):
                _lib.check(L.fl_adjoint(P.handle, 16, ysc.data_ptr(), DTYPES[torch.float32],
                                        xo.data_ptr(), DTYPES[torch.float32], stream.cuda_stream))
        run_fwd(); run_adj()
        _, tf = timed(run_fwd)
        _, ta = timed(run_adj)
        tf /= reps
        ta /= reps
        # adjoint launch = weighting pass + gather kernel; report the gather share via ncu
        b_fwd = n_isect * 4 + n_rays * 4      # f32 voxel gathers + f32 sinogram writes
        b_adj = n_isect * 4 + P.n_vox * 4     # f32 sinogram gathers + f32 voxel writes
        peak = None
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
                peak = json.load(fh).get("hbm_gbs")
            peak_src = "measured"
        except OSError:
            peak, peak_src = 6800.0, "fallback"
        detail.update(n_isect=n_isect, mean_isect_per_ray=n_isect / n_rays,
                      fwd_ms=tf * 1e3, adj_ms=ta * 1e3,
                      fwd_alg_GBps=b_fwd / tf / 1e9, adj_alg_GBps=b_adj / ta / 1e9,
                      fwd_rays_per_s=n_rays / tf, adj_voxel_updates_per_s=n_isect / ta)
        dom = "adjoint" if ta > tf else "forward"
        ach = (b_adj / ta if dom == "adjoint" else b_fwd / tf) / 1e9
        traffic = None
        tpath = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tpath):
            with open(tpath) as fh:
                tj = json.load(fh)
            ent = tj.get(a.workload, {}).get(dom)
            if ent:
                traffic = ent.get("bytes_per_launch")
        roofline = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak if peak else None, "traffic": traffic,
                    "kernel": f"matched {dom} (f32 storage)",
                    "peak_source": peak_src,
                    "bytes_definition": "sum over rays of voxels crossed x element bytes + "
                                        "one element per ray (forward) / per voxel (adjoint)"}
        launches += 0

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cpu = cpu_sample(w, p)

    if rank == 0:
        out = {"metric": metric, "value": value, "unit": "iter/s", "n_gpus": world,
               "steps": K, "warmup": W, "ms_per_step": 1000.0 * t_g / K,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32",
               "data": "synthetic: seeded 12-ellipsoid phantom, noiseless projections",
               "config": config, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
               "clocks": clocks.summary(), "gpu_launches": launches, "detail": detail}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
