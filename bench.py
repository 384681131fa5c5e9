#!/usr/bin/env python
"""Benchmarks of the FrameLab hot path on one GB300.

Default workload ``cone512`` (the headline): 512^3 ellipsoid phantom, 720
views over 2*pi, 1024x768 flat panel at 0.5 mm, source-isocentre 600 mm,
source-detector 1200 mm, 0.5 mm voxels. A step is one CGLS iteration on
(A^T A + lam I) u = b, b = A^T A x_true, with the matched Siddon projector pair:

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

Other workloads (``--workload``), same JSON contract:
* ``cone256`` -- 256^3, 360 views, 512x384 panel at 1 mm (adds the dot-product
  identity and the FP16-storage error to ``detail``); ``cone128`` for profiling;
* ``fan256`` -- 256^2 fan beam, 360 views, 512 bins, SO = OD = 500 mm, 20 CGLS;
* ``fanbatch64`` -- 64 fan slices of uneven size (n in {128..512}, 180..720
  views, 2n bins) with Gaussian noise, batched CGLS (one launch per operator
  for all slices); a step is one iteration of all 64 slices;
* ``sb256`` -- split Bregman (2-level linear framelet, lam 0.01, mu 1, 5 inner
  CGLS) on 256^3 from 90 Poisson-noisy views; a step is one outer iteration.

``--impl reference`` times the reference's CPU path for the workload alone.
Multi-GPU: replicas only (independent solves per rank, no collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

_CONE = dict(SO=600.0, SD=1200.0, lam=0.0)
WORKLOADS = {
    # 512^3 cone CGLS (the large cone-beam configuration)
    "cone512": dict(kind="cone", n=512, nv=720, na=1024, nb=768, det_mm=0.5, vox_mm=0.5, **_CONE),
    # 256^3 circular cone projector pair
    "cone256": dict(kind="cone", n=256, nv=360, na=512, nb=384, det_mm=1.0, vox_mm=1.0, **_CONE),
    # small case for ncu captures
    "cone128": dict(kind="cone", n=128, nv=90, na=256, nb=192, det_mm=2.0, vox_mm=2.0, **_CONE),
    # 2-D fan: 256^2 over a 256 mm field, 360 views, 512 bins, SO = OD = 500 mm
    "fan256": dict(kind="fan", n=256, nv=360, nd=512, SO=500.0, OD=500.0, L=256.0, lam=0.0),
    # 64 uneven fan slices, same scanner, Gaussian noise 1% of each slice's maximum
    "fanbatch64": dict(kind="batch", slices=64, sizes=(128, 192, 256, 384, 512),
                       nv=(180, 720), SO=500.0, OD=500.0, L=256.0, noise=0.01, seed=7),
    # split Bregman on 256^3 from 90 views, Poisson counts at I0 = 1e5
    "sb256": dict(kind="sb", n=256, nv=90, na=512, nb=384, det_mm=1.0, vox_mm=1.0, SO=600.0,
                  SD=1200.0, I0=1e5, pmax=4.0, lam=0.01, mu=1.0, inner=5, levels=2),
    # the same solve on 128^3 (small case for ncu captures of the framelet kernels)
    "sb128": dict(kind="sb", n=128, nv=90, na=256, nb=192, det_mm=2.0, vox_mm=2.0, SO=600.0,
                  SD=1200.0, I0=1e5, pmax=4.0, lam=0.01, mu=1.0, inner=5, levels=2),
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
    ap.add_argument("--symmetry", default="all", choices=["all", "mirror", "none"],
                    help="kernel forms a plan may use: every symmetry its scan has "
                         "(default), the z mirror alone (no half or quarter turn), or none "
                         "(general kernels)")
    ap.add_argument("--only", default="",
                    help="comma list of legs: mixed,plain,hostplain,e2e,kernels,seq,grad,"
                         "parity,dropin")
    return ap.parse_args()


# --------------------------------------------------------------------------
# geometries
# --------------------------------------------------------------------------
def cone_para(w, nv=None):
    from framelab_gb300 import geometry as G
    return G.cone_para_mm(w["n"], nv or w["nv"], w["na"], w["nb"], det_pitch_mm=w["det_mm"],
                          SO_mm=w["SO"], SD_mm=w["SD"], voxel_mm=w["vox_mm"])


def fan_para(n, nv, nd, w):
    """Fan scan of an n x n image over an L x L mm field; the detector spans the
    field's magnified diagonal (2*sqrt(2)*L at magnification 2)."""
    from framelab_gb300 import geometry as G
    L = w["L"]
    return G.fan_para(n, n, nd, nv, L=(L, L), SO=w["SO"], OD=w["OD"],
                      Ly=math.sqrt(2.0) * L * (w["SO"] + w["OD"]) / w["SO"])


def batch_slices(w):
    rng = np.random.default_rng(w["seed"])
    ns = rng.choice(np.array(w["sizes"]), w["slices"])
    nvs = rng.integers(w["nv"][0], w["nv"][1] + 1, w["slices"])
    return [(int(n), int(v)) for n, v in zip(ns, nvs)]


def para_of(w):
    k = w["kind"]
    if k in ("cone", "sb"):
        return cone_para(w)
    if k == "fan":
        return fan_para(w["n"], w["nv"], w["nd"], w)
    return [fan_para(n, v, 2 * n, w) for n, v in batch_slices(w)]


def describe(name, w, world):
    k = w["kind"]
    if k == "cone":
        wl = (f"{name}: {w['n']}^3 cone CGLS, {w['nv']} views, {w['na']}x{w['nb']} panel @ "
              f"{w['det_mm']} mm, SO {w['SO']:.0f} mm, SD {w['SD']:.0f} mm, voxel {w['vox_mm']} mm")
        metric = "CGLS iter/s (cone-beam, matched Siddon pair, fused FP32 graph form)"
        vb, sb = 4 * w["n"] ** 3, 4 * w["nv"] * w["na"] * w["nb"]
        l2 = (f"working set {'>' if 4 * vb + sb > 129e6 else '<'} L2 (4 volume vectors "
              f"{4 * vb / 2**20:.0f} MiB + sinogram {sb / 2**20:.0f} MiB)")
        data = "synthetic: seeded 12-ellipsoid phantom, noiseless projections"
    elif k == "fan":
        wl = (f"{name}: {w['n']}^2 fan CGLS, {w['nv']} views, {w['nd']} bins, "
              f"{w['L']:.0f} mm field, SO {w['SO']:.0f} mm, OD {w['OD']:.0f} mm")
        metric = "CGLS iter/s (fan-beam, matched Siddon pair, fused FP32 graph form)"
        l2 = ("working set < L2 (256 KiB image, 720 KiB sinogram): the L2-resident "
              "case the reference's 2-D configuration is")
        data = "synthetic: seeded 10-ellipse phantom, noiseless projections"
    elif k == "batch":
        wl = (f"{name}: {w['slices']} fan slices, n in {list(w['sizes'])}, "
              f"{w['nv'][0]}..{w['nv'][1]} views, 2n bins, batched CGLS")
        metric = "batched CGLS iter/s (64 uneven fan slices per iteration)"
        l2 = "working set > L2 (4 image-sized vectors + sinogram ~ 0.2 GB)"
        data = ("synthetic: seeded 10-ellipse phantoms, Gaussian noise "
                f"sigma = {w['noise']} x max(sinogram) per slice")
    else:
        wl = (f"{name}: split Bregman, {w['n']}^3, {w['nv']} views, {w['na']}x{w['nb']} "
              f"panel @ {w['det_mm']} mm, {w['levels']}-level linear framelet, "
              f"lam {w['lam']}, mu {w['mu']}, {w['inner']} CGLS per outer iteration")
        metric = "split-Bregman outer iter/s (cone-beam, 2-level linear framelet)"
        nc = 53 * 4 * w["n"] ** 3            # 26 + 27 bands of the 2-level linear framelet
        l2 = f"working set > L2 (framelet coefficients 2 x {nc / 2**30:.2f} GiB)"
        data = (f"synthetic: seeded 12-ellipsoid phantom scaled to max line integral "
                f"{w['pmax']}, Poisson counts at I0 = {w['I0']:.0e}")
    config = {"workload": wl, "global_batch": world, "l2": l2,
              "parallelism": f"replicas{world}"}
    return metric, config, data


# --------------------------------------------------------------------------
# CPU legs: the reference's CPU kernels (oracle restatement, bit-exact)
# --------------------------------------------------------------------------
def _threads():
    return max(1, os.cpu_count() or 1)


def cone_pair_seconds(w, p, row_step=16, av=16):
    """Seconds for one forward (Ax_cone_mf_cpu_siddon) + one backprojection
    (Atx_cone_mf_cpu_new) of the oracle's bit-exact restatement with all host
    threads, from a bounded sample (several seconds of CPU work) extrapolated
    linearly.
    Forward sample: four views per thread, spread over the scan, every
    `row_step`-th detector row (a ray depends only on its view, column and
    row, so these are rays of the full scan). Backprojection sample: one slice
    per thread, spread over z, x `av` views spread over the scan."""
    import concurrent.futures as cf
    import oracle as O
    threads = _threads()
    n, nv, nb = w["n"], len(p["sd_phi"]), w["nb"]
    rng = np.random.default_rng(0)
    x = rng.random(n ** 3, dtype=np.float32)
    fv = min(nv, 4 * threads)
    fsel = np.linspace(0, nv - 1, fv).astype(int)
    rows = np.arange(0, nb, row_step)
    q = dict(p)
    q["sd_phi"] = p["sd_phi"][fsel]
    q["sd_z"] = p["sd_z"][fsel]
    q["z_det"] = p["z_det"][rows]
    q["id_X"] = p["id_X"][fsel]
    t0 = time.perf_counter()
    O.cone_siddon_f32(x, q, threads=threads)
    t_f = time.perf_counter() - t0
    fwd_full = t_f * (nv / fv) * (nb / len(rows))
    av = min(av, nv)
    asel = np.linspace(0, nv - 1, av).astype(int)
    y = rng.random(av * w["na"] * nb, dtype=np.float32)
    r = dict(p)
    for k in ("cos_phi", "sin_phi", "sd_phi", "sd_z"):
        r[k] = p[k][asel]
    r["id_Y"] = np.arange(av, dtype=np.uint32).reshape(av, 1)
    r["Nv"] = np.array([av], np.uint32)
    r["tmp_size"] = np.uint32(av)
    zs = min(threads, n)
    zsel = np.linspace(0, n - 1, zs).astype(int)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda z: O.cone_adj_f32(y, r, threads=1, slices=(int(z), int(z) + 1)), zsel))
    t_a = time.perf_counter() - t0
    adj_full = t_a * (n / zs) * (nv / av)
    desc = (f"Ax_cone_mf_cpu_siddon on {fv}/{nv} views x {len(rows)}/{nb} rows ({t_f:.2f} s) + "
            f"Atx_cone_mf_cpu_new on {zs}/{n} slices x {av}/{nv} views ({t_a:.2f} s)")
    return fwd_full + adj_full, desc


def fan_pair_seconds(p, views=None):
    """Seconds for one fan forward (Ax_fan_mf_cpu_siddon) + backprojection
    (Atx_fan_mf_cpu_new), oracle restatement, all host threads; with `views`,
    on that many views of the scan, extrapolated to all of them."""
    import oracle as O
    from framelab_gb300 import geometry as G
    threads = _threads()
    nv = len(p["sd_phi"])
    q = p
    if views and views < nv:
        nx, nd = int(p["nx"]), len(p["y_det"])
        sd = p["sd_phi"][np.linspace(0, nv - 1, views).astype(int)]
        q = G.fan_para(nx, nx, nd, views, sd_phi=sd)
        for k in ("SO", "OD", "scale", "y_det", "cos_det", "sin_det", "dy_det"):
            q[k] = p[k]
    rng = np.random.default_rng(0)
    nx, ny = int(q["nx"]), int(q["ny"])
    x = rng.random(nx * ny, dtype=np.float32)
    y = rng.random(len(q["sd_phi"]) * len(q["y_det"]), dtype=np.float32)
    t0 = time.perf_counter()
    O.fan_siddon_f32(x, q, threads=threads)
    O.fan_adj_f32(y, q, threads=threads)
    t = time.perf_counter() - t0
    return t * nv / len(q["sd_phi"])


def framelet_seconds(w, block=64):
    """Seconds for one framelet analysis + synthesis of the sb workload's
    volume: the FP64 numpy restatement on a block^3 volume, scaled by voxels."""
    from oracle import numerics as N
    rng = np.random.default_rng(0)
    u = rng.random((block,) * 3)
    t0 = time.perf_counter()
    c = N.frame_dec(u, w["levels"], "linear")
    N.frame_rec(c, "linear")
    t = time.perf_counter() - t0
    return t * (w["n"] / block) ** 3, t


def cpu_sample(w, p):
    threads = _threads()
    k = w["kind"]
    if k == "cone":
        s, desc = cone_pair_seconds(w, p)
        return dict(value=1.0 / s, unit="iter/s", cores=threads, kind="port",
                    sample=f"{desc}, {threads} threads, extrapolated linearly to one forward + "
                           f"backprojection ({s:.0f} s per CGLS iteration)")
    if k == "fan":
        s = fan_pair_seconds(p)
        return dict(value=1.0 / s, unit="iter/s", cores=threads, kind="port",
                    sample=f"Ax_fan_mf_cpu_siddon + Atx_fan_mf_cpu_new on the full scan, "
                           f"{threads} threads ({s:.2f} s per CGLS iteration)")
    if k == "batch":
        sl = batch_slices(w)
        pick = sorted(range(len(sl)), key=lambda i: sl[i][0])[::4]   # sizes spread
        tot, smp = 0.0, 0.0
        per = {}
        for i in pick:
            n, v = sl[i]
            t = fan_pair_seconds(p[i], views=min(v, 128))
            per[n] = per.get(n, []) + [t / v]                       # seconds per view
            smp += t * min(v, 128) / v
        for n, v in sl:
            near = min(per, key=lambda m: abs(m - n))
            tot += statistics.mean(per[near]) * v * (n / near) ** 2
        return dict(value=1.0 / tot, unit="iter/s", cores=threads, kind="port",
                    sample=f"Ax_fan_mf_cpu_siddon + Atx_fan_mf_cpu_new on 128 views of "
                           f"{len(pick)} of {len(sl)} slices ({smp:.1f} s), {threads} threads, "
                           f"scaled per slice by views and pixels ({tot:.1f} s per iteration)")
    s, desc = cone_pair_seconds(w, p, row_step=4, av=16)
    tf, t64 = framelet_seconds(w)
    it = w["inner"] * s + tf
    return dict(value=1.0 / it, unit="iter/s", cores=threads, kind="port",
                sample=f"{w['inner']} x ({desc}) + framelet analysis/synthesis on 64^3 "
                       f"({t64:.2f} s, numpy) scaled by voxels; {threads} threads "
                       f"({it:.0f} s per outer iteration)")


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

    def busy(self, step, min_samples=2, max_s=10.0):
        """Run untimed warm-up steps until the sampler has seen the GPU under
        load (min_samples readings, or max_s seconds), so that a timed region
        shorter than the 200 ms sampling period still has clocks beside it."""
        if not self.proc:
            return
        t0 = time.perf_counter()
        n0 = len(self.rows)
        import torch
        while len(self.rows) - n0 < min_samples and time.perf_counter() - t0 < max_s:
            step()
            torch.cuda.synchronize()

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
# GPU legs
# --------------------------------------------------------------------------
def max_over_ranks(t: float, world: int, device) -> float:
    """The slowest replica's time: the job ends when every rank has."""
    if world > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([t], device=device, dtype=torch.float64)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        return float(x.item())
    return t


def job_rate(world: int, steps: int, t_max: float) -> float:
    """Whole-job throughput of independent replicas (weak scaling): every rank
    does `steps` steps, all of them done after t_max seconds."""
    return world * steps / t_max


class Ctx:
    """Device, stream, replica bookkeeping and the CUDA-event timer."""

    def __init__(self, a, world, rank, local):
        import torch
        self.torch = torch
        self.a, self.world, self.rank, self.local = a, world, rank, local
        self.dev = torch.device("cuda", local)
        self.stream = torch.cuda.current_stream()
        self.K, self.W = a.steps, a.warmup
        self.legs = (set(a.only.split(",")) if a.only else
                     {"mixed", "plain", "hostplain", "e2e", "kernels", "seq", "grad", "parity",
                      "dropin"})

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def tmax(self, t):
        return max_over_ranks(t, self.world, self.dev)

    def timed(self, fn):
        """Run fn between CUDA events on the launching stream, synchronised and
        barriered on both sides; returns (result, max-over-ranks seconds)."""
        torch = self.torch
        self.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(self.stream)
        out = fn()
        e1.record(self.stream)
        torch.cuda.synchronize()
        self.barrier()
        return out, self.tmax(e0.elapsed_time(e1) / 1000.0)

    def rel(self, a_, b_):
        t = self.torch
        return (t.linalg.vector_norm((a_ - b_).double()) /
                t.linalg.vector_norm(b_.double())).item()


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh).get("hbm_gbs"), "measured"
    except OSError:
        return 6800.0, "fallback"


def roofline_model(form):
    """Per-intersection counts of one kernel form's pair ("refl4": quarter turns
    with the reflection, "oct": quarter turns), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_model.json")) as fh:
            m = json.load(fh)
    except OSError:
        return None
    k = m.get("forms", {}).get(form)
    if not k:
        return None
    return dict(k, sms=m["sms"], l1_wavefronts_per_sm_cycle=m["l1_wavefronts_per_sm_cycle"],
                issue_per_sm_cycle=m["issue_per_sm_cycle"])


def projector_roofline(ctx, workload, n_isect, n_rays, n_vox, t_fwd, t_adj, detail, label,
                       sm_mhz=None, l1_form=None):
    """The dominant projector kernel against the bound it runs into.

    The matched projectors gather every voxel / sinogram value a ray or voxel
    needs through L1 (the algorithmic bytes below move at 1.3-1.9x the HBM
    copy rate, so they are L1/L2 hits, not DRAM traffic). With l1_form the
    roofline is the L1 data pipe: wavefronts per intersection from the ncu
    capture of the kernel form in use (profiles/roofline_model.json) times this
    workload's intersections, over the CUDA-event time, against 1 wavefront
    per SM-cycle at the SM clock sampled during the run. Issue slots and the
    HBM fraction of the compulsory bytes (input read once, output written
    once) stand beside it; so does the algorithmic-bytes figure."""
    b_fwd = n_isect * 4 + n_rays * 4      # f32 voxel gathers + f32 sinogram writes
    b_adj = n_isect * 4 + n_vox * 4       # f32 sinogram gathers + f32 voxel writes
    peak, src = hbm_peak()
    detail.update(n_isect=n_isect, mean_isect_per_ray=n_isect / n_rays,
                  fwd_ms=t_fwd * 1e3, adj_ms=t_adj * 1e3,
                  fwd_alg_GBps=b_fwd / t_fwd / 1e9, adj_alg_GBps=b_adj / t_adj / 1e9,
                  fwd_rays_per_s=n_rays / t_fwd, adj_voxel_updates_per_s=n_isect / t_adj)
    dom = "adjoint" if t_adj > t_fwd else "forward"
    t = t_adj if dom == "adjoint" else t_fwd
    compulsory = 4 * (n_rays + n_vox)     # one pass over the input and the output
    alg = (b_adj if dom == "adjoint" else b_fwd)
    hbm = {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": src,
           "compulsory_GBps": compulsory / t / 1e9,
           "compulsory_frac": compulsory / t / 1e9 / peak if peak else None,
           "algorithmic_GBps": alg / t / 1e9,
           "algorithmic_frac": alg / t / 1e9 / peak if peak else None}
    m = roofline_model(l1_form) if l1_form else None
    if not m:
        # no per-intersection L1 model for this kernel form: the DRAM view of
        # the compulsory bytes, with the gather bytes (served by L1 / L2)
        # beside it -- those exceed what HBM could deliver, so they are no
        # roofline
        return {"bound": "hbm", "achieved": compulsory / t / 1e9, "peak": peak, "unit": "GB/s",
                "frac": compulsory / t / 1e9 / peak if peak else None, "traffic": None,
                "kernel": f"{label} {dom} (f32 storage)", "peak_source": src,
                "bytes_definition": "compulsory: one element per ray and per voxel "
                                    "(input read once, output written once)",
                "gathers_served_by_l1_l2": {
                    "GBps": alg / t / 1e9,
                    "bytes_definition": "sum over rays of voxels crossed x element bytes + "
                                        "one element per ray (forward) / per voxel (adjoint)"},
                "note": "latency / issue / L1 bound (profiles/ for the counters)"}
    k = m[dom]
    f = (sm_mhz or 2070.0) * 1e6
    sms = m["sms"]
    ach = k["l1_wavefronts_per_isect"] * n_isect / t
    pk = m["l1_wavefronts_per_sm_cycle"] * sms * f
    iss = k["warp_inst_per_isect"] * n_isect / t
    ipk = m["issue_per_sm_cycle"] * sms * f
    return {"bound": "l1", "achieved": ach, "peak": pk, "unit": "wavefronts/s",
            "frac": ach / pk, "traffic": k["dram_bytes_per_isect"] * n_isect,
            "kernel": f"{label} {dom} ({k['kernel']})",
            "peak_source": f"1 L1 data-pipe wavefront per SM-cycle x {sms} SMs x "
                           f"{f / 1e6:.0f} MHz (SM clock sampled in this run)",
            "model": "ncu per-intersection counts of the kernel form in use at cone256 "
                     "(profiles/roofline_model.json) x this workload's intersections; "
                     "traffic likewise scaled (a lower bound at larger sizes, where L2 "
                     "reuse across views falls)",
            "issue": {"achieved": iss, "peak": ipk, "unit": "warp-instructions/s",
                      "frac": iss / ipk},
            "hbm": hbm}


def time_pair(ctx, P, x, reps=3):
    """CUDA-event seconds of one matched forward and one matched adjoint."""
    from framelab_gb300 import _lib
    from framelab_gb300.projector import DTYPES
    torch = ctx.torch
    L = _lib.load()
    s = ctx.stream.cuda_stream
    y = torch.empty(P.n_rays, device=ctx.dev, dtype=torch.float32)
    xo = torch.empty(P.n_vox, device=ctx.dev, dtype=torch.float32)
    f32 = DTYPES[torch.float32]

    def fwd():
        for _ in range(reps):
            _lib.check(L.fl_forward(P.handle, 16, x.data_ptr(), f32, y.data_ptr(), f32, s))

    def adj():
        for _ in range(reps):
            _lib.check(L.fl_adjoint(P.handle, 16, y.data_ptr(), f32, xo.data_ptr(), f32, s))
    fwd(); adj()
    _, tf = ctx.timed(fwd)
    _, ta = ctx.timed(adj)
    return tf / reps, ta / reps, y, xo


def host_structure_cgls(ctx, P, b, lam, cg_g, detail, iters=2):
    """The reference's plain FP32 GPU structure with this library's projectors:
    solveCGLS.m (u0 = 0) with its algebra on host FP32 arrays (FP32 inner
    products, as MATLAB's on single arrays), and every A / A^T call through
    host buffers -- its input copied to the device and its output back, as
    the reference's mex GPU projectors do for MATLAB arrays. Timed over
    `iters` iterations after one untimed."""
    import time
    torch = ctx.torch
    bh = b.cpu().numpy().astype(np.float32)

    def normal(v):
        y = P.forward(torch.from_numpy(v).to(ctx.dev)).cpu()
        q = P.adjoint(y.to(ctx.dev)).reshape(-1).cpu().numpy()
        return q + np.float32(lam) * v if lam else q

    def cgls(n):
        u = np.zeros_like(bh)
        r = bh.copy()
        p = r.copy()
        gamma = float(np.dot(r, r))
        for _ in range(n):
            q = normal(p)
            alpha = gamma / float(np.dot(p, q))
            u += np.float32(alpha) * p
            r -= np.float32(alpha) * q
            g1 = float(np.dot(r, r))
            p = r + np.float32(g1 / gamma) * p
            gamma = g1
        return u

    cgls(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = cgls(iters)
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / iters
    u_ref = cg_g.solve(b, lam=lam, iters=iters).reshape(-1).cpu().numpy()
    out = {"host_structure_iter_per_s": 1.0 / t,
           "host_structure_vs_graph_rel_l2": float(np.linalg.norm(u - u_ref) /
                                                   max(np.linalg.norm(u_ref), 1e-30)),
           "graph_over_host_structure": detail["graph_iter_per_s_per_gpu"] * t}
    if "mixed_iter_per_s" in detail:
        out["mixed_over_host_structure"] = detail["mixed_iter_per_s"] * t
    return out


def parity_block(ctx, w, p):
    """Parity of the matched pair on this workload's own geometry (the oracle
    as the checker, untimed): the plan with its half / quarter turns and the
    plan without them, each against the FP64 exact model, beside the
    reference's own FP32 CPU kernels against the same model. Cone volumes on
    seeded subsets (20,000 rays; 2,000 or 4,000 voxels), fans in full
    (oracle/parity.py)."""
    torch = ctx.torch
    import oracle.parity as PAR
    from framelab_gb300 import phantoms as PH
    from framelab_gb300.projector import Plan
    n = w["n"]
    x = PH.ellipsoids_3d(n, seed=1) if w["kind"] == "cone" else PH.ellipses_2d(n, seed=1)
    out = {}
    for form in ("turns", "precise"):
        P = Plan(p)
        if form == "precise":
            P.quarter_turn = False
            P.rot_mirror = False
            P.reflect = False
        t = P.views_per_walk

        def fwd(v, P=P):
            return P.forward(torch.from_numpy(np.ascontiguousarray(v)).to(ctx.dev)).cpu().numpy()

        def adj(v, P=P):
            return P.adjoint(torch.from_numpy(np.ascontiguousarray(v)).to(ctx.dev)).cpu().numpy()
        t0 = time.perf_counter()
        if w["kind"] == "cone":
            r = PAR.cone_parity(p, x, fwd, adj, n_rays=20000, n_vox=2000 if n >= 512 else 4000,
                                turns=P.rotations, reflect=P.reflect)
        else:
            r = PAR.fan_parity(p, x, fwd, adj, turns=P.rotations, reflect=P.reflect)
        r["views_per_walk"] = t
        r["seconds"] = time.perf_counter() - t0
        out[form] = r
        del P
        torch.cuda.empty_cache()
    return out


def dropin_pair(ctx, w, p):
    """The MATLAB classes' path: version 1 (ConeBeamScanner/setPara.m:82), i.e.
    Ax_cone_mf_gpu_new + Atx_cone_mf_gpu_new through host pointers, as
    ConeBeamScanner/apply.m and applyAdjoint.m call them -- each call copies
    its input to the device and its output back (the bit-exact replicas of
    the reference's CPU kernels). Wall-clock seconds of one call each, after
    one untimed pair."""
    import ctypes as C
    from framelab_gb300 import _lib
    L = _lib.load()
    n, na, nb = w["n"], w["na"], w["nb"]
    nv = len(p["sd_phi"])
    rng = np.random.default_rng(0)
    X = rng.random(n ** 3, dtype=np.float32)
    y = np.zeros(nv * na * nb, np.float32)
    yn = np.zeros_like(y)
    Y = rng.random(nv * na * nb, dtype=np.float32)
    xo = np.zeros(n ** 3, np.float32)
    a = {k: np.ascontiguousarray(p[k], np.float32)
         for k in ("sd_phi", "sd_z", "y_det", "z_det", "cos_phi", "sin_phi")}
    idY = np.ascontiguousarray(np.asarray(p["id_Y"]).T.reshape(-1).astype(np.int32))
    Nv = np.ascontiguousarray(p["Nv"].astype(np.int32))
    P_ = lambda v: v.ctypes.data_as(C.c_void_p)
    nvb, ts = int(p["nv_block"]), int(p["tmp_size"])

    def fwd():
        L.Ax_cone_mf_gpu_new(P_(X), P_(y), P_(yn), P_(a["sd_phi"]), P_(a["sd_z"]), P_(a["y_det"]),
                             P_(a["z_det"]), P_(idY), P_(Nv), float(p["SO"]), float(p["OD"]),
                             float(p["scale"]), float(p["dz"]), n, n, n, 1, na, nb, nv, ts, nvb)
        _lib.check_last()

    def adj():
        L.Atx_cone_mf_gpu_new(P_(xo), P_(Y), P_(a["cos_phi"]), P_(a["sin_phi"]), P_(a["sd_z"]),
                              P_(a["y_det"]), P_(a["z_det"]), P_(idY), P_(Nv), float(p["SO"]),
                              float(p["OD"]), float(p["scale"]), float(p["dy_det"]),
                              float(p["y_os"]), float(p["dz_det"]), float(p["dz"]), n, n, n, 1,
                              na, nb, nv, ts, nvb)
        _lib.check_last()
    fwd(); adj()
    ctx.torch.cuda.synchronize()
    t0 = time.perf_counter(); fwd(); t1 = time.perf_counter(); adj(); t2 = time.perf_counter()
    return {"dropin_iter_per_s": 1.0 / (t2 - t0), "dropin_forward_s": t1 - t0,
            "dropin_adjoint_s": t2 - t1,
            "dropin_call": "Ax_cone_mf_gpu_new + Atx_cone_mf_gpu_new (host pointers, version 1)",
            "dropin_bytes_copied_per_iter": 4 * (2 * n ** 3 + 3 * nv * na * nb)}


def restrict_symmetry(ctx, P):
    """--symmetry: keep the plan to the z mirror alone, or to the general
    kernels (the default uses every symmetry the scan has)."""
    if ctx.a.symmetry in ("mirror", "none"):
        P.rot_mirror = False
    if ctx.a.symmetry == "none":
        P.z_mirror = False


def run_single(ctx, name, w, p):
    """cone / fan: CGLS on one scan (graph headline, mixed, plain, e2e, kernels)."""
    torch = ctx.torch
    from framelab_gb300 import phantoms as PH
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS, dot
    K, W, world = ctx.K, ctx.W, ctx.world
    P = Plan(p)
    restrict_symmetry(ctx, P)
    shapes = P.autotune()                 # launch shapes for this geometry (untimed)
    n = w["n"]
    img = PH.ellipsoids_3d(n, seed=5) if w["kind"] == "cone" else PH.ellipses_2d(n, seed=5)
    x_true = torch.from_numpy(img.reshape(-1)).to(ctx.dev)
    f = P.forward(x_true)
    b = P.adjoint(f).reshape(-1)
    del f
    torch.cuda.synchronize()
    lam = w["lam"]
    detail = {"launch_shapes": shapes}
    cg_g = NativeCGLS(P, "graph")
    if W:
        cg_g.solve(b, lam=lam, iters=W)
    clocks = ClockSampler(ctx.local)
    with clocks:
        clocks.busy(lambda: cg_g.solve(b, lam=lam, iters=max(W, 1)))
        u_g, t_g = ctx.timed(lambda: cg_g.solve(b, lam=lam, iters=K))
    detail["graph_iter_per_s_per_gpu"] = K / t_g
    detail["graph_vs_truth_rel_l2"] = ctx.rel(u_g, x_true)
    if "mixed" in ctx.legs:
        cg_m = NativeCGLS(P, "mixed")
        if W:
            cg_m.solve(b, lam=lam, iters=W, refresh=REFRESH)
        u_m, t_m = ctx.timed(lambda: cg_m.solve(b, lam=lam, iters=K, refresh=REFRESH))
        detail["mixed_iter_per_s"] = world * K / t_m
        detail["mixed_vs_graph_rel_l2"] = ctx.rel(u_m, u_g)
        del cg_m, u_m
    if "plain" in ctx.legs:
        cg_p = NativeCGLS(P, "plain")
        if W:
            cg_p.solve(b, lam=lam, iters=W)
        u_p, t_p = ctx.timed(lambda: cg_p.solve(b, lam=lam, iters=K))
        detail["plain_iter_per_s"] = world * K / t_p
        detail["graph_over_plain"] = t_p / t_g
        detail["mixed_over_plain"] = (detail["mixed_iter_per_s"] / detail["plain_iter_per_s"]
                                      if "mixed_iter_per_s" in detail else None)
        detail["graph_vs_plain_rel_l2"] = ctx.rel(u_g, u_p)
        del cg_p, u_p
    if "hostplain" in ctx.legs:
        detail.update(host_structure_cgls(ctx, P, b, lam, cg_g, detail))
    e2e = None
    if "e2e" in ctx.legs:
        bh = torch.empty(b.numel(), dtype=torch.float32, pin_memory=True)
        bh.copy_(b.cpu())
        uh = torch.zeros(b.numel(), dtype=torch.float32, pin_memory=True)
        bn, un = bh.numpy(), uh.numpy()
        cg_g.solve_host(bn, un, lam=lam, iters=max(W, 1))
        _, t_e = ctx.timed(lambda: cg_g.solve_host(bn, un, lam=lam, iters=K))
        nb = b.numel() * 4
        e2e = {"value": world * K / t_e, "unit": "iter/s",
               "h2d_bytes_per_step": nb / K, "d2h_bytes_per_step": nb / K,
               "call": f"fl_cgls_solve_host, {K} iterations per call: b in, u out "
                       "(pinned host buffers, read and written in place by the fold "
                       "kernels over the host link; u0 = 0 needs no transfer)"}
    roofline = None
    if "kernels" in ctx.legs:
        cnt = P.count_intersections()
        n_isect = int(cnt.sum(dtype=torch.int64).item())
        del cnt
        p32 = (u_g / (u_g.abs().max() + 1e-30)).contiguous()
        tf, ta, y, xo = time_pair(ctx, P, p32)
        roofline = projector_roofline(ctx, name, n_isect, P.n_rays, P.n_vox, tf, ta, detail,
                                      "matched", clocks.summary().get("sm_mhz"),
                                      l1_form=({(4, True): "refl4", (4, False): "oct"}
                                               .get((P.rotations, P.reflect))
                                               if w["kind"] == "cone" else None))
        if w["kind"] == "cone":
            # dot-product identity <A x, y> = <x, A^T y> on N(0,1) vectors (FP64 dots)
            g = torch.Generator(device=ctx.dev).manual_seed(11)
            xr = torch.randn(P.n_vox, device=ctx.dev, generator=g)
            yr = torch.randn(P.n_rays, device=ctx.dev, generator=g)
            lhs = dot(P.forward(xr), yr)
            rhs = dot(xr, P.adjoint(yr))
            detail["dot_test_rel"] = abs(lhs - rhs) / abs(lhs)
            # FP16 storage of the volume against FP32 storage (same kernel)
            y32 = P.forward(x_true)
            y16 = P.forward(x_true.half())
            detail["fp16_storage_vs_fp32_rel_l2"] = ctx.rel(y16, y32)
            del xr, yr, y32, y16
    if "parity" in ctx.legs:
        detail["parity"] = parity_block(ctx, w, p)
    if "dropin" in ctx.legs and w["kind"] == "cone":
        detail.update(dropin_pair(ctx, w, p))
    if "grad" in ctx.legs and w["kind"] == "cone":
        # gradient of 1/2 |A x - b|^2 through the autograd binding (backward =
        # the exact-transpose backprojector) against central differences on 64
        # random voxels, h = 1e-3, at the CGLS iterate
        from framelab_gb300.autograd import fd_gradcheck
        f = P.forward(x_true)
        t0 = time.perf_counter()
        err, _ = fd_gradcheck(P, u_g.reshape(-1), f, n_vox=64, h=1e-3)
        detail["gradcheck_max_rel_err"] = err
        detail["gradcheck_voxels"] = 64
        detail["gradcheck_s"] = time.perf_counter() - t0
        del f
    return dict(value=job_rate(world, K, t_g), t_step=t_g / K, e2e=e2e, roofline=roofline,
                # ncu-checked: 5 per iteration (a fan plan's forward adds its
                # transposed copy: 6), the start, and the z fold / unfold
                launches=(5 if P.cone else 6) * K + 1 + (2 if P.z_mirror else 0), detail=detail,
                clocks=clocks.summary(), unit="iter/s")


def run_batch(ctx, name, w, paras):
    """fanbatch: batched CGLS over uneven fan slices (one launch per operator and
    kind of slice: general, or half / quarter turn)."""
    torch = ctx.torch
    from framelab_gb300 import phantoms as PH
    from framelab_gb300.batch import FanBatch
    from framelab_gb300.solvers import NativeCGLS
    K, W, world = ctx.K, ctx.W, ctx.world
    B = FanBatch(paras)
    parts = B.autotune()                  # parts per walked ray of the turn slices (untimed)
    x_true = B.concat_images([PH.ellipses_2d(P.nx, seed=100 + i)
                              for i, P in enumerate(B.plans)]).to(ctx.dev)
    sino = B.forward(x_true)
    g = torch.Generator(device=ctx.dev).manual_seed(w["seed"])
    for s in B.sinograms(sino):
        s += w["noise"] * s.max() * torch.randn(s.shape, device=ctx.dev, generator=g)
    rhs = B.adjoint(sino)
    del sino
    torch.cuda.synchronize()
    detail = {"slices": len(B), "n_vox": B.n_vox, "n_rays": B.n_rays,
              "slices_by_rays_per_walk": {str(t): B.turns.count(t) for t in (1, 2, 4, 8)},
              "reflection_slices": sum(B.reflect),
              "turn_parts_per_ray": parts}
    if W:
        B.cgls(rhs, iters=W)
    clocks = ClockSampler(ctx.local)
    with clocks:
        clocks.busy(lambda: B.cgls(rhs, iters=max(W, 1)))
        u, t_b = ctx.timed(lambda: B.cgls(rhs, iters=K))
    detail["slice_iter_per_s"] = len(B) * K / t_b
    detail["vs_truth_rel_l2"] = ctx.rel(u, x_true)
    if "seq" in ctx.legs:
        # the same solves one slice after another (one plan + CGLS per slice)
        sols = [NativeCGLS(P, "graph") for P in B.plans]
        parts = [r.reshape(-1).contiguous() for r in B.images(rhs)]
        for cg, r in zip(sols, parts):
            cg.solve(r, iters=max(W, 1))
        us, t_s = ctx.timed(lambda: [cg.solve(r, iters=K) for cg, r in zip(sols, parts)])
        detail["sequential_iter_per_s"] = K / t_s
        detail["batched_over_sequential"] = t_s / t_b
        detail["batched_vs_sequential_rel_l2"] = ctx.rel(u, torch.cat(us))
        del sols, us
    e2e = None
    if "e2e" in ctx.legs:
        rh = torch.empty(B.n_vox, dtype=torch.float32, pin_memory=True)
        rh.copy_(rhs.cpu())
        uh = torch.empty(B.n_vox, dtype=torch.float32, pin_memory=True)

        def host_solve():
            r = rh.to(ctx.dev, non_blocking=True)
            uh.copy_(B.cgls(r, iters=K), non_blocking=True)
        host_solve()
        _, t_e = ctx.timed(host_solve)
        nb = B.n_vox * 4
        e2e = {"value": world * K / t_e, "unit": "iter/s",
               "h2d_bytes_per_step": nb / K, "d2h_bytes_per_step": nb / K,
               "call": f"FanBatch.cgls, {K} iterations per call: right-hand sides in "
                       "(pinned host), solutions out"}
    roofline = None
    if "kernels" in ctx.legs:
        n_isect = sum(int(P.count_intersections().sum(dtype=torch.int64).item())
                      for P in B.plans)
        xs = (u / (u.abs().max() + 1e-30)).contiguous()
        reps = 3
        y = B.forward(xs)
        xo = B.adjoint(y)
        _, tf = ctx.timed(lambda: [B.forward(xs, out=y) for _ in range(reps)])
        _, ta = ctx.timed(lambda: [B.adjoint(y, out=xo) for _ in range(reps)])
        roofline = projector_roofline(ctx, name, n_isect, B.n_rays, B.n_vox, tf / reps,
                                      ta / reps, detail, "batched matched")
    return dict(value=job_rate(world, K, t_b), t_step=t_b / K, e2e=e2e, roofline=roofline,
                launches=B.launches_per_iteration * K + 1, detail=detail,
                clocks=clocks.summary(), unit="iter/s")


def run_sb(ctx, name, w, p):
    """sb: split Bregman outer iterations (5 CGLS + framelet step each)."""
    torch = ctx.torch
    from framelab_gb300 import phantoms as PH
    from framelab_gb300.projector import Plan
    from framelab_gb300.transforms import SplitBregmanSolver
    K, W, world = ctx.K, ctx.W, ctx.world
    P = Plan(p)
    restrict_symmetry(ctx, P)
    shapes = P.autotune()                 # launch shapes for this geometry (untimed)
    x = torch.from_numpy(PH.ellipsoids_3d(w["n"], seed=5).reshape(-1)).to(ctx.dev)
    proj = P.forward(x)
    s = w["pmax"] / float(proj.max())
    x_phys = x * s
    g = torch.Generator(device=ctx.dev).manual_seed(3)
    counts = torch.poisson(w["I0"] * torch.exp(-proj * s), generator=g)
    f = -torch.log(counts.clamp(min=1.0) / w["I0"])
    del proj, counts
    u0 = torch.zeros(P.n_vox, device=ctx.dev)
    kw = dict(lam=w["lam"], mu=w["mu"], cg_iters=w["inner"])
    # the workspace (framelet, CGLS, coefficient sets) is allocated once, as
    # for the CGLS workloads; each step is one outer iteration of solve()
    sbs = SplitBregmanSolver(P, levels=w["levels"], kind="linear", mode="graph")
    detail = {"launch_shapes": shapes}
    if W:
        sbs.solve(f, u0, outer=W, **kw)
    clocks = ClockSampler(ctx.local)
    with clocks:
        clocks.busy(lambda: sbs.solve(f, u0, outer=max(W, 1), **kw))
        u, t_s = ctx.timed(lambda: sbs.solve(f, u0, outer=K, **kw))
    hist = sbs.history
    detail["vs_truth_rel_l2"] = ctx.rel(u, x_phys)
    detail["last_relative_update"] = float(hist[-1]) if len(hist) else None
    e2e = None
    if "e2e" in ctx.legs:
        fh = torch.empty(f.numel(), dtype=torch.float32, pin_memory=True)
        fh.copy_(f.reshape(-1).cpu())
        uh = torch.empty(P.n_vox, dtype=torch.float32, pin_memory=True)

        def host_solve():
            fd = fh.to(ctx.dev, non_blocking=True).view_as(f)
            uh.copy_(sbs.solve(fd, u0, outer=K, **kw), non_blocking=True)
        _, t_e = ctx.timed(host_solve)
        e2e = {"value": world * K / t_e, "unit": "iter/s",
               "h2d_bytes_per_step": f.numel() * 4 / K, "d2h_bytes_per_step": P.n_vox * 4 / K,
               "call": f"SplitBregmanSolver.solve (fl_sb_run), {K} outer iterations per call: "
                       "sinogram in (pinned host), volume out"}
    roofline = None
    if "kernels" in ctx.legs:
        cnt = P.count_intersections()
        n_isect = int(cnt.sum(dtype=torch.int64).item())
        del cnt
        tf, ta, _, _ = time_pair(ctx, P, (u / (u.abs().max() + 1e-30)).contiguous())
        roofline = projector_roofline(ctx, name, n_isect, P.n_rays, P.n_vox, tf, ta, detail,
                                      "matched")
        # one framelet step of the outer loop (analysis with shrink and Bregman
        # update, synthesis into b), against its compulsory bytes: u read, b
        # written, v read and written, t written and read back
        from framelab_gb300.transforms import FrameletSystem
        fw = FrameletSystem((w["n"],) * 3, "linear", w["levels"])
        v = torch.zeros(fw.ncoef, device=ctx.dev)
        t = torch.empty_like(v)
        bb = torch.empty_like(u)
        fw.bregman(u, v, t, None, w["mu"], w["lam"] / w["mu"], bb)
        reps = 3
        _, tfw = ctx.timed(lambda: [fw.bregman(u, v, t, None, w["mu"], w["lam"] / w["mu"], bb)
                                    for _ in range(reps)])
        tfw /= reps
        fw.fused = False                # the separable pass per axis, for comparison
        fw.bregman(u, v, t, None, w["mu"], w["lam"] / w["mu"], bb)
        _, tsep = ctx.timed(lambda: [fw.bregman(u, v, t, None, w["mu"], w["lam"] / w["mu"], bb)
                                     for _ in range(reps)])
        tsep /= reps
        fw.fused = True
        fb = 4 * (2 * P.n_vox + 4 * fw.ncoef)
        detail.update(framelet_step_ms=tfw * 1e3, framelet_compulsory_GBps=fb / tfw / 1e9,
                      framelet_separable_step_ms=tsep * 1e3, framelet_ncoef=fw.ncoef)
        del v, t, bb, fw
    # setup: A^T f (packing + gather) and W u0 (1 per level); per outer iteration:
    # fold b and u, warm-start residual (fwd, adj, + mu u) + init, inner x (fwd,
    # adj, 3 updates), unfold u; Bregman analysis + synthesis (1 + 2 per level);
    # |u_k - u_{k-1}| (diff, 2 dots). Checked against an ncu launch list of one
    # call (sb128, 4 outer iterations: 168 launches).
    launches = 2 + w["levels"] + K * (7 + 5 * w["inner"] + 3 * w["levels"] + 3)
    return dict(value=job_rate(world, K, t_s), t_step=t_s / K, e2e=e2e, roofline=roofline,
                launches=launches, detail=detail, clocks=clocks.summary(), unit="iter/s")


# --------------------------------------------------------------------------
def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[a.workload]
    metric, config, data = describe(a.workload, w, world)
    if a.symmetry != "all":
        config["symmetry"] = a.symmetry

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
               "cpu_baseline": {"value": v, "unit": "iter/s",
                                "cores": samples[0]["cores"] if samples else None,
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
    ctx = Ctx(a, world, rank, local)
    p = para_of(w)
    run = {"cone": run_single, "fan": run_single, "batch": run_batch, "sb": run_sb}[w["kind"]]
    res = run(ctx, a.workload, w, p)

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cpu = cpu_sample(w, p)

    if rank == 0:
        out = {"metric": metric, "value": res["value"], "unit": res["unit"], "n_gpus": world,
               "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000.0 * res["t_step"],
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": data, "config": config, "e2e": res["e2e"],
               "roofline": res["roofline"], "cpu_baseline": cpu, "clocks": res["clocks"],
               "gpu_launches": res["launches"], "detail": res["detail"]}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
