"""Benchmark: Msamples/s of the 1080p textured-heightfield workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (seeded synthetic data, see cudart_gb300/scenes.py large_textured):
1024x1024-vertex heightfield (~2.09M triangles) with a 1024^2 RGBA8 texture,
64 glass/mirror icospheres, 4 quad lights; 1920x1080, 256 samples per pixel,
max depth 8.  One step renders the whole frame (531M path samples).

* value: wavefront form, device time (CUDA events on the render stream),
  scene resident in HBM; L2 flushed (256 MiB write) before every step.
* plain_kernel: the drop-in megakernel on the same frame, timed on both
  node formats (8-bit quantised and FP32) and reported on the faster one;
  its accumulator must equal the wavefront's bit for bit (equal RMSE by
  construction).
* e2e: the public API from host arrays to host image: crt_scene_create
  (BVH build + uploads) + crt_render_create + crt_render_pass +
  crt_render_resolve, wall clock.
* roofline: the dominant stage of a profiled pass (per-launch CUDA events,
  node and triangle fetches counted by an untimed re-run) against the L2
  gather ceiling measured live by crt_measure_gather (node- and triangle-
  sized records at random indices of a 64 MiB working set, L2 only); its
  DRAM part (ncu traffic per ray) against the measured HBM copy bandwidth.
* cpu_baseline / --impl reference: the CPU oracle port of the reference's
  `--cpu` path on all host threads over a bounded pixel sample.

Under torchrun each rank renders its own sample range of one frame (rank r:
samples [r*spp, (r+1)*spp), weak scaling) and the step ends with one sum of
the ranks' FP32 accumulators (NCCL all_reduce), the only exchange.

The JSON line carries the contract's keys first and the headline's own
figures last; per-stage timings, the autotuner's candidates and the
inversion's details go to a second file, bench_detail.json (in the
directory named by --detail-dir, default the working directory).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Msamples/s at 1080p, equal RMSE, vs plain kernel; adjoint/forward time ratio"
WORKLOAD = ("large_textured 1920x1080 256spp depth8: 1024^2-vertex heightfield + 1024^2 RGBA8 "
            "texture, 64 glass/mirror icospheres (subdiv 3), 4 quad lights, 2,174,986 triangles")
NODE_BYTES, F32_NODE_BYTES, TRI_BYTES = 80, 208, 48
L2_FLUSH_BYTES = 256 << 20


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def gather_ceiling(torch, stream, record_sizes, working_set=64 << 20, l1=False, loads=256, repeats=5):
    """GB/s of random record gathers (crt_measure_gather) from a working set
    of `working_set` bytes (64 MiB: resident in L2, half its size; 96 KiB:
    resident in every SM's L1 when l1): one figure per record size, best of
    `repeats` launches of 1216 blocks x 256 threads (8 per SM on 152 SMs),
    each thread fetching `loads` records.  Bytes = records x size."""
    from cudart_gb300 import measure_gather
    buf = torch.ones(working_set // 4, dtype=torch.float32, device="cuda")
    n_threads = 1216 * 256
    out = {}
    for rb in record_sizes:
        measure_gather(buf, rb, n_threads, 8, l1=l1, stream=stream.cuda_stream)   # warm: data into L2
        best = None
        for _ in range(repeats):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            measure_gather(buf, rb, n_threads, loads, l1=l1, stream=stream.cuda_stream)
            e.record(stream)
            e.synchronize()
            ms = s.elapsed_time(e)
            best = ms if best is None else min(best, ms)
        out[rb] = n_threads * loads * rb / (best * 1e-3) / 1e9
    del buf
    return out


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def cpu_port_sample(sc, seconds: float, threads: int):
    """Oracle port (restatement of the reference's --cpu path) and a bounded
    sample of the frame sized to about `seconds` of work on `threads`:
    a stratified pixel subset at 1 spp, or the whole frame at k spp.
    Returns (scene, camera, pixels, spp)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle
    oracle.build()
    o = oracle.OracleScene(sc)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    npix = sc.width * sc.height
    probe = (np.arange(4096, dtype=np.uint64) * (npix // 4096) % npix).astype(np.uint32)
    t = time.perf_counter()
    o.render(cam, 7, 1, sc.max_depth, pixels=probe, threads=threads)
    rate = len(probe) / max(time.perf_counter() - t, 1e-6)
    target = max(4096.0, rate * seconds)
    if target <= npix:
        n = int(target)
        px = (np.arange(n, dtype=np.uint64) * (npix // n) % npix).astype(np.uint32)
        return o, cam, px, 1
    return o, cam, None, int(round(target / npix))


def run_reference(args):
    """--impl reference: the CPU path timed on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from cudart_gb300 import scenes
    threads = os.cpu_count() or 1
    sc = scenes.large_textured()
    o, cam, px, k_spp = cpu_port_sample(sc, 5.0, threads)
    n_samples = (len(px) if px is not None else sc.width * sc.height) * k_spp
    times = []
    for k in range(args.warmup + args.steps):
        t = time.perf_counter()
        o.render(cam, 1234, k_spp, sc.max_depth, pixels=px, spp0=k * k_spp, threads=threads)
        if k >= args.warmup:
            times.append(time.perf_counter() - t)
    dt = sum(times)
    value = n_samples * args.steps / dt / 1e6
    sample = (f"{n_samples} samples per step: "
              + (f"{len(px)} stratified pixels x 1 spp" if px is not None else f"full frame x {k_spp} spp")
              + " of the 1920x1080 frame")
    print(json.dumps({
        "metric": METRIC, "value": round(value, 5), "unit": "Msamples/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * dt / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": WORKLOAD, "path": "CPU restatement of the reference --cpu path, OpenMP"},
        "cpu_baseline": {"value": round(value, 5), "unit": "Msamples/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 5), "unit": "Msamples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)


def batched_views_leg(args, torch, stream):
    """C4: the 64 views of the batched-views generator over the mixed scene
    in one wavefront batch (autotuned launch options incl. BVH width) against
    the same views as 64 sequential plain-kernel renders.  spp / spp_div per
    view keeps the leg to a few seconds; both arms render the same samples."""
    import dataclasses
    from cudart_gb300 import GB300Batch, GB300Scene, autotune, options_dict, scenes
    sc = scenes.mixed_mid()
    views = [dataclasses.replace(v, spp=max(1, v.spp // args.c4_spp_div))
             for v in scenes.batched_views(base=sc).views]
    samples = sum(v.width * v.height * v.spp for v in views)
    g = GB300Scene(sc)
    t0 = time.perf_counter()
    tune = autotune(g, 1024, 1024, max_depth=sc.max_depth, trial_spp=16, repeats=2, rounds=1,
                    tune_bvh_width=True)
    tune_s = time.perf_counter() - t0
    opts = tune.options
    out = {"workload": f"mixed_mid (102,412 triangles), 64 views r=12, resolutions "
                       f"{{256^2, 512^2, 768x432, 1024^2}}, spp {{16, 64, 256}} / {args.c4_spp_div}, depth 8",
           "samples_per_step": samples,
           "autotuned": {k: v for k, v in options_dict(opts).items() if k not in ("seed", "max_depth", "view_id")},
           "bvh_width": tune.bvh_width, "tune_seconds": round(tune_s, 2),
           "tune_candidates": tune.candidates}
    res = {}
    # the plain kernel on each node format; the faster one is the comparator
    for name, kw in (("batched_wavefront", dict(options=opts)),
                     ("sequential_plain_q8", dict(mode="megakernel", node_format="q8")),
                     ("sequential_plain_f32", dict(mode="megakernel", node_format="f32"))):
        b = GB300Batch(g, views, max_depth=sc.max_depth, **kw)
        b.set_stream(stream.cuda_stream)
        b.render_pass(1)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        t_host = time.perf_counter()
        b.render()
        host_ms = (time.perf_counter() - t_host) * 1e3   # the host has queued every wave
        e.record(stream)
        torch.cuda.synchronize()
        ms = s.elapsed_time(e)
        res[name] = {"ms": round(ms, 2), "msamples_per_s": round(samples / (ms * 1e-3) / 1e6, 2),
                     "host_enqueue_ms": round(host_ms, 2)}
        del b
    plain = max(("sequential_plain_q8", "sequential_plain_f32"), key=lambda k: res[k]["msamples_per_s"])
    res["sequential_plain"] = dict(res[plain], node_format=plain.rsplit("_", 1)[1])
    out.update(res)
    out["speedup"] = round(res["batched_wavefront"]["msamples_per_s"] / res["sequential_plain"]["msamples_per_s"], 3)
    return out


def config_legs(args, torch, stream):
    """The two other single-frame workloads at their own sizes: the Cornell
    box (512^2, 16 spp, depth 5, 36 triangles) and the mixed-material scene
    (1280x720, 128 spp, depth 8, 102,412 triangles).  Each frame on the
    wavefront form (autotuned on the frame, BVH width included) and on the
    plain kernel (faster node format), best of 3 after a warm-up, L2 flushed
    before each; accumulators must agree bit for bit."""
    import numpy as np
    from cudart_gb300 import GB300Renderer, GB300Scene, autotune, scenes
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    out = {}
    for name, sc in (("cornell_512", scenes.cornell_box()), ("mixed_720p", scenes.mixed_mid())):
        g = GB300Scene(sc)
        spp = sc.spp
        tune = autotune(g, sc.width, sc.height, max_depth=sc.max_depth, trial_spp=min(16, spp), repeats=2,
                        rounds=1, tune_bvh_width=True)
        opts = tune.options
        opts.seed, opts.view_id = 1234, 0
        rs = {"wavefront": GB300Renderer(g, sc.width, sc.height, spp, options=opts)}
        for fmt in ("q8", "f32"):
            rs["plain_" + fmt] = GB300Renderer(g, sc.width, sc.height, spp, max_depth=sc.max_depth, seed=1234,
                                               mode="megakernel", node_format=fmt)
        ms, acc = {}, {}
        for k, r in rs.items():
            r.set_stream(stream.cuda_stream)
            best = None
            for rep in range(4):
                flush.fill_(float(rep))
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                r.reset()
                s.record(stream)
                r.render(spp)
                e.record(stream)
                e.synchronize()
                if rep:
                    best = s.elapsed_time(e) if best is None else min(best, s.elapsed_time(e))
            ms[k] = best
            acc[k] = r.accum()
        plain = min(("plain_q8", "plain_f32"), key=lambda k: ms[k])
        n = sc.width * sc.height * spp
        out[name] = {"value": round(n / (ms["wavefront"] * 1e-3) / 1e6, 1),
                     "plain": round(n / (ms[plain] * 1e-3) / 1e6, 1),
                     "vs_plain": round(ms[plain] / ms["wavefront"], 3),
                     "identical": bool(all(np.array_equal(acc["wavefront"], a) for a in acc.values())),
                     "bvh_width": tune.bvh_width}
        del rs, g
    return out


def adjoint_leg(args, torch, stream):
    """C5: Cornell shell + 32 boxes at 512^2, 64 spp per iteration, depth 6.
    adjoint/forward: one adjoint pass (primal trace + replay, both on the GPU)
    against one forward wavefront pass of the same 64 spp (CUDA events, median
    of 5).  Then the material inversion: target 1024 spp with the true
    albedos, start at albedo 0.5 for the 32 boxes, L2 loss on the image
    clamped to [0, 1] (the displayed range), Adam at
    lr 1e-2 for `inversion_iters` iterations, gradients from the adjoint on
    samples independent of the iteration's image (the same samples would
    correlate the residual with its derivative and bias the gradient)."""
    import numpy as np
    from cudart_gb300 import GB300Renderer, GB300Scene, scenes
    sc = scenes.material_inversion()
    g = GB300Scene(sc)
    n_mats = len(sc.materials)
    kd_true = np.array([m.kd for m in sc.materials], np.float32)
    boxes = np.arange(4, n_mats)
    npix = sc.width * sc.height
    r = GB300Renderer(g, sc.width, sc.height, sc.spp, max_depth=sc.max_depth, seed=77, mode="wavefront")
    r.set_stream(stream.cuda_stream)
    # target image: 1024 spp with the true albedos (its own sample range)
    r.restart(1 << 24)
    r.render(1024)
    target = torch.from_numpy(r.accum()).cuda() / 1024
    adj = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    gkd = torch.zeros((n_mats, 3), dtype=torch.float32, device="cuda")
    gka = torch.zeros((n_mats, 3), dtype=torch.float32, device="cuda")
    adj[:, :3] = 1.0
    fw, bw = [], []
    for k in range(6):
        r.restart(k * sc.spp)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        r.render(sc.spp)
        e.record(stream)
        s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s2.record(stream)
        r.adjoint(k * sc.spp, sc.spp, adj.data_ptr(), gkd.data_ptr(), gka.data_ptr())
        e2.record(stream)
        torch.cuda.synchronize()
        if k:
            fw.append(s.elapsed_time(e))
            bw.append(s2.elapsed_time(e2))
    f_ms, a_ms = statistics.median(fw), statistics.median(bw)
    out = {"workload": "material_inversion: Cornell shell + 32 diffuse boxes (396 triangles), "
                       "512x512, 64 spp, depth 6",
           "forward_ms": round(f_ms, 3), "adjoint_ms": round(a_ms, 3), "ratio": round(a_ms / f_ms, 3),
           "roulette": "survival probability held constant (unbiased gradient of the expected image)"}
    out["inversion"] = run_inversion(torch, g, r, sc, target, kd_true, boxes, args.inversion_iters,
                                     loss=args.inversion_loss, exact=False)
    vis = box_visibility(torch, g, sc, boxes)
    err = np.array(out["inversion"]["albedo_rmse_per_box"])
    seen = vis >= 100
    out["inversion"]["visible_pixels_per_box"] = vis.tolist()
    out["inversion"]["albedo_rmse_end_visible"] = (round(float(np.sqrt(np.mean(err[seen] ** 2))), 4)
                                                   if seen.any() else None)
    out["inversion"]["visible_boxes"] = int(seen.sum())
    return out


def box_visibility(torch, g, sc, mats):
    """Pixels whose centre's camera ray first hits each material in `mats`
    (pinhole camera of the scene; crt_trace_closest)."""
    import numpy as np
    from cudart_gb300 import camera_from_json
    c = camera_from_json(sc.camera, sc.width, sc.height)
    eye, d, up, right = (np.array(v[:], np.float64) for v in (c.eye, c.dir, c.up, c.right))
    ys, xs = np.mgrid[0:sc.height, 0:sc.width]
    nx = (2.0 * (xs + 0.5) / sc.width - 1.0).ravel()
    ny = (1.0 - 2.0 * (ys + 0.5) / sc.height).ravel()
    dirs = d[None] + right[None] * (c.fov * c.aspect) * nx[:, None] + up[None] * c.fov * ny[:, None]
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays = np.zeros((len(dirs), 8), np.float32)
    rays[:, :3] = eye
    rays[:, 3] = 1e-5
    rays[:, 4:7] = dirs
    rays[:, 7] = np.finfo(np.float32).max
    face, _, _ = g.trace_closest(torch.from_numpy(rays).cuda())
    face = face.cpu().numpy()
    ids = np.asarray(sc.material_ids).astype(np.int64)
    mat = np.where(face >= 0, ids[np.maximum(face, 0)], -1)
    return np.array([int(np.sum(mat == m)) for m in mats])


def run_inversion(torch, g, r, sc, target, kd_true, boxes, iters, loss="clamped", exact=False,
                  snr_evals=8):
    """Adam (lr 1e-2) on the box albedos from 0.5, one 64-spp render and one
    adjoint on independent samples per iteration.  loss "clamped": L2 on the
    image clamped to [0, 1] (gradient zero where the estimate saturates);
    "masked": L2 on the radiance over the pixel-channels where the target is
    below 1; "hdr": plain L2 on the radiance.  exact: exact-roulette adjoint.  Also
    the gradient's signal-to-noise ratio per box at the start (mean over
    `snr_evals` independent adjoints / their spread)."""
    import numpy as np
    n_mats = len(sc.materials)
    npix = sc.width * sc.height
    adj = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    gkd = torch.zeros((n_mats, 3), dtype=torch.float32, device="cuda")
    gka = torch.zeros((n_mats, 3), dtype=torch.float32, device="cuda")
    kd = kd_true.copy()
    kd[boxes] = 0.5
    m1 = np.zeros_like(kd)
    m2 = np.zeros_like(kd)
    b1, b2, lr, eps = 0.9, 0.999, 1e-2, 1e-8
    err0 = float(np.sqrt(np.mean((kd[boxes] - kd_true[boxes]) ** 2)))

    def grad_at(kd_vals, it, spp0_adj):
        g.set_materials(kd=kd_vals)
        r.restart(it * sc.spp)
        r.render(sc.spp)
        img = torch.from_numpy(r.accum()).cuda() / sc.spp
        if loss == "clamped":
            diff = img.clamp(0, 1) - target.clamp(0, 1)
            adj[:, :3] = 2.0 * diff * (img < 1).float() / sc.spp
        elif loss == "masked":
            # L2 over the pixel-channels the target does not saturate: the
            # mask is fixed, so no noisy estimate decides which terms count
            diff = (img - target) * (target < 1).float()
            adj[:, :3] = 2.0 * diff / sc.spp
        else:
            diff = img - target
            adj[:, :3] = 2.0 * diff / sc.spp
        gkd.zero_()
        gka.zero_()
        r.adjoint(spp0_adj, sc.spp, adj.data_ptr(), gkd.data_ptr(), gka.data_ptr(), exact_roulette=exact)
        r.synchronize()
        return float((diff ** 2).sum()), gkd.cpu().numpy()

    def image_loss(kd_vals):
        """L2 image loss of a 1024-spp render (its own sample range) against
        the target: the optimisation's progress without the noise of one
        64-spp iteration."""
        g.set_materials(kd=kd_vals)
        r.restart(1 << 25)   # not the target's samples (1 << 24) nor the iterations'
        r.render(1024)
        img = torch.from_numpy(r.accum()).cuda() / 1024
        if loss == "clamped":
            return float(((img.clamp(0, 1) - target.clamp(0, 1)) ** 2).sum())
        if loss == "masked":
            return float((((img - target) * (target < 1).float()) ** 2).sum())
        return float(((img - target) ** 2).sum())

    # gradient SNR at the start point: independent 64-spp adjoints
    gs = np.array([grad_at(kd, 10000 + k, (1 << 22) + k * sc.spp)[1][boxes] for k in range(snr_evals)])
    snr = np.abs(gs.mean(0)) / np.maximum(gs.std(0, ddof=1), 1e-30)
    clean0 = image_loss(kd)
    losses = []
    t0 = time.perf_counter()
    for it in range(iters):
        loss_v, grad = grad_at(kd, it, (1 << 23) + it * sc.spp)
        losses.append(loss_v)
        grad[np.setdiff1d(np.arange(n_mats), boxes)] = 0.0
        m1 = b1 * m1 + (1 - b1) * grad
        m2 = b2 * m2 + (1 - b2) * grad * grad
        step = lr * (m1 / (1 - b1 ** (it + 1))) / (np.sqrt(m2 / (1 - b2 ** (it + 1))) + eps)
        kd = np.clip(kd - step, 0.01, 0.99).astype(np.float32)
    seconds = round(time.perf_counter() - t0, 2)
    clean1 = image_loss(kd)
    g.set_materials(kd=kd_true)
    box_err = np.sqrt(np.mean((kd[boxes] - kd_true[boxes]) ** 2, axis=1))
    q = max(1, min(20, len(losses) // 4))
    return {"iterations": iters, "lr": lr, "loss": loss, "exact_roulette": exact,
            "loss_median_first_iters": round(float(np.median(losses[:q])), 4),
            "loss_median_last_iters": round(float(np.median(losses[-q:])), 4),
            "image_loss_1024spp_start": round(clean0, 4), "image_loss_1024spp_end": round(clean1, 4),
            "albedo_rmse_start": round(err0, 4),
            "albedo_rmse_end": round(float(np.sqrt(np.mean(box_err ** 2))), 4),
            "albedo_rmse_per_box": [round(float(x), 4) for x in box_err],
            "grad_snr_per_box_start": [round(float(x), 3) for x in np.median(snr, axis=1)],
            "seconds": seconds}


def inversion_study(args):
    """Material-inversion variants on the C5 workload: loss clamped / HDR,
    constant-survival / exact-roulette adjoint; per-box errors, visibility
    and gradient SNR.  One JSON line."""
    import numpy as np
    import torch
    from cudart_gb300 import GB300Renderer, GB300Scene, scenes
    sc = scenes.material_inversion()
    g = GB300Scene(sc)
    kd_true = np.array([m.kd for m in sc.materials], np.float32)
    boxes = np.arange(4, len(sc.materials))
    r = GB300Renderer(g, sc.width, sc.height, sc.spp, max_depth=sc.max_depth, seed=77, mode="wavefront")
    r.set_stream(torch.cuda.current_stream().cuda_stream)   # torch's adjoint buffers and the adjoint: one stream
    r.restart(1 << 24)
    r.render(1024)
    target = torch.from_numpy(r.accum()).cuda() / 1024
    vis = box_visibility(torch, g, sc, boxes)
    out = {"visible_pixels_per_box": vis.tolist(), "variants": []}
    for loss, exact in (("clamped", False), ("masked", False), ("hdr", False), ("clamped", True), ("masked", True)):
        res = run_inversion(torch, g, r, sc, target, kd_true, boxes, args.inversion_iters, loss, exact)
        err = np.array(res["albedo_rmse_per_box"])
        for thr in (100, 1000):
            m = vis >= thr
            res[f"albedo_rmse_end_visible_{thr}px"] = round(float(np.sqrt(np.mean(err[m] ** 2))), 4) if m.any() else None
        out["variants"].append(res)
    print(json.dumps(out), flush=True)


def run_gb300(args):
    import numpy as np
    import torch
    from cudart_gb300 import GB300Renderer, GB300Scene, autotune, options_dict, scenes
    from cudart_gb300.sharding import reduce_accumulators, sample_range

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    spp = args.spp
    sc = scenes.large_textured(spp=spp) if not args.small else scenes.large_textured(
        width=480, height=270, spp=spp, grid=256, tex_size=256, n_spheres=16)
    npix = sc.width * sc.height
    # one non-default stream carries the renders, the L2 flushes and the events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    scene = GB300Scene(sc)
    info = scene.info
    # launch options: the autotuner on this frame (untimed; BVH width kept at
    # 8, the 4-wide tree of this scene measured slower)
    tuned = None
    if not args.no_tune:
        t0 = time.perf_counter()
        tune = autotune(scene, sc.width, sc.height, max_depth=sc.max_depth, trial_spp=64, repeats=2,
                        rounds=1, tune_bvh_width=False)
        tuned = {"options": {k: v for k, v in options_dict(tune.options).items()
                             if k not in ("seed", "max_depth", "view_id")},
                 "candidates": tune.candidates, "seconds": round(time.perf_counter() - t0, 2),
                 "start_ms_per_spp": round(tune.start_ms_per_spp, 3),
                 "tuned_ms_per_spp": round(tune.ms_per_spp, 3)}
        opts = tune.options
        opts.seed, opts.view_id = 1234, 0
        wf = GB300Renderer(scene, sc.width, sc.height, spp, options=opts)
    else:
        # --options sets launch options by hand (e.g. to profile one variant)
        extra = json.loads(args.options) if args.options else {}
        wf = GB300Renderer(scene, sc.width, sc.height, spp, max_depth=sc.max_depth, seed=1234,
                           mode="wavefront", **extra)
    wf.set_stream(stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    # this rank's samples of the frame: [s0, s0 + spp) of world * spp
    s0, s1 = sample_range(world * spp, rank, world)
    assert s1 - s0 == spp

    def step(r):
        r.restart(s0)
        r.render(spp)
        if dist is not None:
            reduce_accumulators(r.accum_tensor())

    def timed_steps(r, k_steps):
        durs = []
        for k in range(k_steps):
            flush.fill_(float(k))
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            step(r)
            e.record(stream)
            durs.append((s, e))
        torch.cuda.synchronize()
        return [s.elapsed_time(e) for s, e in durs]

    for _ in range(args.warmup):
        step(wf)
    barrier()
    with ClockSampler(local) as clk:
        barrier()
        ms = timed_steps(wf, args.steps)
        barrier()
    clocks = clk.summary()
    ms_step = sum(ms) / len(ms)
    if dist is not None:
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    value = world * npix * spp / (ms_step * 1e-3) / 1e6
    ext, shd = wf.ray_counts()          # counters restart at every reset: last step only
    rays_per_sample = (ext + shd) / (npix * spp)
    wf_acc = wf.accum()

    # plain drop-in megakernel on the same frame, on whichever node format
    # it runs faster (each timed after one warm-up frame)
    k_plain = max(1, min(args.steps, 2))
    plain_by_format = {}
    identical = True
    for fmt in ("q8", "f32"):
        mk = GB300Renderer(scene, sc.width, sc.height, spp, max_depth=sc.max_depth, seed=1234,
                           mode="megakernel", node_format=fmt)
        mk.set_stream(stream.cuda_stream)
        step(mk)
        torch.cuda.synchronize()
        plain_by_format[fmt] = sum(timed_steps(mk, k_plain)) / k_plain
        identical = identical and bool(np.array_equal(mk.accum(), wf_acc))
        del mk
    plain_fmt = min(plain_by_format, key=plain_by_format.get)
    mk_ms = plain_by_format[plain_fmt]
    plain_value = npix * spp / (mk_ms * 1e-3) / 1e6

    out = None
    detail = {}
    if rank == 0:
        # roofline: profiled pass of 8 spp (per-launch events, counted fetches)
        prof_r = GB300Renderer(scene, sc.width, sc.height, spp, options=wf.options)
        prof_r.set_stream(stream.cuda_stream)
        prof = prof_r.profile_pass(8)
        stages = ("generate", "extend", "shade", "shadow", "accumulate", "bookkeeping")
        dom = max(stages, key=lambda s: prof[f"{s}_ms"])
        peak, peak_kind = measured_peaks()
        node_bytes = NODE_BYTES if wf.options.node_format != 1 else F32_NODE_BYTES
        roof = {}
        # algorithmic bytes of the gathers: visits to the nodes staged in
        # shared memory (top_nodes) are counted apart, not as L1/L2 gathers
        for stage, rays, nodes, tris, top in (
                ("extend", "extension_rays", "extension_nodes", "extension_tris", "extension_top_nodes"),
                ("shadow", "shadow_rays", "shadow_nodes", "shadow_tris", "shadow_top_nodes")):
            launches = prof[f"{stage}_launches"]
            alg = (prof[nodes] - prof[top]) * node_bytes + prof[tris] * TRI_BYTES
            ms_l = prof[f"{stage}_ms"] / launches
            gbs = alg / launches / (ms_l * 1e-3) / 1e9
            roof[stage] = {"kernel": "wf_" + stage, "bytes_per_launch": alg / launches,
                           "ms_per_launch": ms_l, "gbs": gbs, "rays": prof[rays],
                           "nodes_per_ray": prof[nodes] / max(prof[rays], 1),
                           "staged_nodes_per_ray": prof[top] / max(prof[rays], 1),
                           "shared_memory_bytes_per_launch": prof[top] * node_bytes / launches,
                           "tris_per_ray": prof[tris] / max(prof[rays], 1)}
        main = roof["extend"] if dom != "shadow" else roof["shadow"]
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic_per_ray.json")
        if os.path.exists(tp):
            fmt = "f32" if wf.options.node_format == 1 else "q8"
            tr = json.load(open(tp)).get(main["kernel"], {}).get(fmt)
            if tr:
                traffic = round(tr["dram_bytes_per_ray"] * main["rays"] / prof[f"{dom if dom in roof else 'extend'}_launches"])
        # the ceiling of the bytes counted: random gathers of node- and
        # triangle-sized records (crt_measure_gather, fetched through L1 as
        # the traversal's loads are) from an L1-resident (96 KiB) and an
        # L2-resident (64 MiB) working set, combined with the traversal's own
        # L1 sector hit rate (ncu, profiles/wf_extend_cache.json):
        # 1 / (h1 / BW_L1 + (1 - h1) / BW_L2), weighted by the byte mix
        ext_k = main["kernel"] == "wf_extend"
        nb = (prof["extension_nodes" if ext_k else "shadow_nodes"]
              - prof["extension_top_nodes" if ext_k else "shadow_top_nodes"]) * node_bytes
        tb = prof["extension_tris" if ext_k else "shadow_tris"] * TRI_BYTES
        g1 = gather_ceiling(torch, stream, (node_bytes, TRI_BYTES), working_set=96 << 10, l1=True)
        g2 = gather_ceiling(torch, stream, (node_bytes, TRI_BYTES), working_set=64 << 20, l1=True)
        mix = lambda g: (nb + tb) / (nb / g[node_bytes] + tb / g[TRI_BYTES])
        bw1, bw2 = mix(g1), mix(g2)
        h1, h1_src = None, None
        cp = os.path.join(ROOT, "profiles", "wf_extend_cache.json")
        if os.path.exists(cp):
            fmt = "f32" if wf.options.node_format == 1 else "q8"
            ent = json.load(open(cp)).get(fmt, {})
            if "l1_sector_hit" in ent:
                h1, h1_src = float(ent["l1_sector_hit"]), "profiles/wf_extend_cache.json"
        hier = 1.0 / (h1 / bw1 + (1.0 - h1) / bw2) if h1 is not None else bw2
        dram_gbs = traffic / (main["ms_per_launch"] * 1e-3) / 1e9 if traffic else None
        roofline = {"bound": "l1+l2 gather" if h1 is not None else "l2 gather", "kernel": main["kernel"],
                    "achieved": round(main["gbs"], 1), "peak": round(hier, 1), "unit": "GB/s",
                    "frac": round(main["gbs"] / hier, 4), "traffic": traffic,
                    "peak_kind": "measured live: crt_measure_gather, L1-resident and L2-resident working sets, "
                                 f"{node_bytes} B node / 48 B triangle records by the byte mix, combined at the "
                                 f"ncu L1 sector hit rate {h1} ({h1_src})",
                    "l2_only": {"peak": round(bw2, 1), "frac": round(main["gbs"] / bw2, 4)},
                    "hbm": {"achieved": round(dram_gbs, 1) if dram_gbs else None, "peak": peak,
                            "frac": round(dram_gbs / peak, 4) if dram_gbs else None,
                            "peak_kind": f"{peak_kind} HBM copy; achieved = ncu DRAM traffic / time"},
                    "limiter": "divergent dependent gathers: see profiles/wf_extend_large_textured_1080p.md "
                               "(issue-active, SIMT lanes, long-scoreboard stalls)",
                    "algorithmic_bytes": f"nodes visited outside the shared-memory top nodes x {node_bytes} B "
                                         "+ triangles tested x 48 B per ray",
                    "staged_nodes_per_ray": round(main["staged_nodes_per_ray"], 3)}
        l2_peak = hier
        step_bytes = None
        if main["kernel"] == "wf_extend":
            # per-step cross-check: all traversal bytes of a step / its time
            per_ray_ext = ((roof["extend"]["nodes_per_ray"] - roof["extend"]["staged_nodes_per_ray"]) * node_bytes
                           + roof["extend"]["tris_per_ray"] * TRI_BYTES)
            per_ray_shd = ((roof["shadow"]["nodes_per_ray"] - roof["shadow"]["staged_nodes_per_ray"]) * node_bytes
                           + roof["shadow"]["tris_per_ray"] * TRI_BYTES)
            step_bytes = ext * per_ray_ext + shd * per_ray_shd
            roofline["step_check"] = {"traversal_bytes_per_step": round(step_bytes),
                                      "gbs_over_whole_step": round(step_bytes / (ms_step * 1e-3) / 1e9, 1),
                                      "within_ceiling": bool(step_bytes / (ms_step * 1e-3) / 1e9 <= l2_peak)}
        detail["roofline"] = {
            "gather_l1_resident_gbs": {str(k): round(v, 1) for k, v in g1.items()},
            "gather_l2_resident_gbs": {str(k): round(v, 1) for k, v in g2.items()},
            "stage_ms": {s_: round(prof[f"{s_}_ms"], 2) for s_ in stages},
            "profile_spp": 8,
            "extend_rays_by_bounce": prof["extend_rays_by_bounce"][:sc.max_depth],
            "extend_ms_by_bounce": [round(x, 3) for x in prof["extend_ms_by_bounce"][:sc.max_depth]],
            "stages": {k: {kk: (round(vv, 3) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                       for k, v in roof.items()}}
        del prof_r

        # e2e: host arrays -> host image through the public API, with the BVH
        # built on the device (the fastest path from arrays to pixels) and,
        # for comparison, on the host
        # what crt_scene_create copies up: positions, normals, uvs, material
        # ids, RGBA8 texels (the material and light tables are a few KB)
        h2d = int(sc.positions.nbytes + sc.normals.nbytes + sc.uvs.nbytes + 4 * sc.n_tris +
                  sum(4 * img.shape[0] * img.shape[1] for img in sc.textures))

        # the step's inputs and its output image live in pinned host memory
        def pinned(a):
            t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0].copy()).dtype, pin_memory=True)
            t.numpy()[...] = a
            return t.numpy()

        sc_pinned = dataclasses.replace(sc, positions=pinned(sc.positions), normals=pinned(sc.normals),
                                        uvs=pinned(sc.uvs), material_ids=pinned(sc.material_ids),
                                        textures=[pinned(img) for img in sc.textures])
        img_out = pinned(np.zeros((sc.height, sc.width, 4), np.uint8))

        def e2e_run(builder):
            e2e_t, create_t, build_t = [], [], []
            for k in range(1 + max(1, min(args.steps, 2))):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s2 = GB300Scene(sc_pinned, builder=builder)
                t1 = time.perf_counter()
                r2 = GB300Renderer(s2, sc.width, sc.height, spp, options=wf.options)
                r2.render(spp)
                img = r2.copy_image_bytes(out=img_out)
                e2e_t.append(time.perf_counter() - t0)
                create_t.append(t1 - t0)
                build_t.append(s2.info.build_ms * 1e-3)
                del r2, s2
            e2e_s = statistics.mean(e2e_t[1:])
            return e2e_s, statistics.mean(create_t[1:]), statistics.mean(build_t[1:]), int(img.nbytes)

        gpu_s, gpu_create, gpu_build, d2h = e2e_run("gpu")
        host_s, host_create, host_build, _ = e2e_run("host")
        e2e = {"value": round(npix * spp / gpu_s / 1e6, 3), "unit": "Msamples/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "seconds_per_step": round(gpu_s, 4),
               "scene_create_s": round(gpu_create, 4),
               "region": "crt_scene_create from pinned host arrays (positions, normals, uvs, ids, RGBA8 "
                         "texture up; records packed and the BVH built on the GPU) + "
                         "crt_render_create + crt_render_pass(256) + crt_render_resolve to host RGBA8",
               "with_host_bvh_build": {"value": round(npix * spp / host_s / 1e6, 3),
                                       "seconds_per_step": round(host_s, 4),
                                       "scene_create_s": round(host_create, 4),
                                       "scene_build_s": round(host_build, 4)}}

        c4 = batched_views_leg(args, torch, stream) if world == 1 and not args.no_extra else None
        c12 = config_legs(args, torch, stream) if world == 1 and not args.no_extra else None
        c5 = adjoint_leg(args, torch, stream) if world == 1 and not args.no_extra else None

        cpu = None
        if world == 1 and not args.no_cpu:
            threads = os.cpu_count() or 1
            o, cam, px, k_spp = cpu_port_sample(sc, 12.0, threads)
            n_samples = (len(px) if px is not None else npix) * k_spp
            t0 = time.perf_counter()
            o.render(cam, 1234, k_spp, sc.max_depth, pixels=px, threads=threads)
            dt = time.perf_counter() - t0
            cpu = {"value": round(n_samples / dt / 1e6, 5), "unit": "Msamples/s", "cores": threads,
                   "kind": "port",
                   "sample": (f"{len(px)} stratified pixels x 1 spp" if px is not None
                              else f"full frame x {k_spp} spp") + f" of the 1920x1080 frame, {dt:.1f} s"}
        cap = wf.options.wave_paths or default_wave_paths(npix)
        waves = math.ceil(spp / max(1, cap // npix)) if npix <= cap else spp * math.ceil(npix / cap)
        # per wave: generate, accumulate, next-wave; per bounce: extend, shade,
        # shadow and the queue switch, plus the shadow-counter reset of the
        # overlapped schedule (once per bounce; the serial one folds it in)
        serial = bool(wf.options.flags & 8)
        launches = args.steps * waves * (3 + (4 if serial else 5) * sc.max_depth)
        if tuned:
            detail["autotune"] = tuned
            tuned = {"options": tuned["options"], "seconds": tuned["seconds"]}
        if c4:
            detail["batched_views"] = c4
            c4 = {k: c4[k] for k in ("speedup", "batched_wavefront", "sequential_plain", "samples_per_step",
                                     "bvh_width", "workload")}
        if c5:
            detail["adjoint"] = c5
            inv = c5["inversion"]
            c5 = {k: c5[k] for k in ("forward_ms", "adjoint_ms", "ratio")}
            c5["inversion"] = {k: inv[k] for k in ("iterations", "albedo_rmse_start", "albedo_rmse_end",
                                                   "albedo_rmse_end_visible", "image_loss_1024spp_start",
                                                   "image_loss_1024spp_end") if k in inv}
        detail["e2e"] = e2e
        e2e = {k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step",
                                   "seconds_per_step")}
        detail["roofline_line"] = dict(roofline)
        roofline = {k: roofline[k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac",
                                             "traffic", "l2_only", "hbm", "step_check", "staged_nodes_per_ray")
                    if k in roofline}
        roofline["hbm"] = {k: roofline["hbm"][k] for k in ("achieved", "peak", "frac")}
        if c4:
            c4 = {"speedup": c4["speedup"],
                  "batched_msamples_per_s": c4["batched_wavefront"]["msamples_per_s"],
                  "sequential_plain_msamples_per_s": c4["sequential_plain"]["msamples_per_s"],
                  "spp_div": args.c4_spp_div}
        # the standard keys first, the headline's own figures last: a reader
        # of the line's last 1500 characters sees them whole
        out = {
            "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator)", "gpu_launches": launches,
            "config": {"workload": "large_textured 1920x1080 256spp depth8, 2,174,986 triangles",
                       "spp": spp, "max_depth": sc.max_depth, "bvh_nodes": info.num_nodes,
                       "sharded": "sample ranges + all_reduce" if world > 1 else None,
                       "l2": "flushed before every step (256 MiB write)"},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks, "e2e": e2e,
            "mrays_per_s": round(value * rays_per_sample, 1),
            "adjoint": c5, "batched_views": c4, "configs": c12,
            "plain_kernel": {"value": round(plain_value, 3), "node_format": plain_fmt,
                             "identical": identical},
            "adjoint_forward_ratio": c5["ratio"] if c5 else None,
            "speedup_vs_plain": round(value / world / plain_value, 3),
        }
        detail["line_extra"] = {"rays_per_sample": round(rays_per_sample, 3), "autotune": tuned,
                                "plain_ms_per_step_by_node_format": {k: round(v, 3) for k, v in plain_by_format.items()},
                                "workload": WORKLOAD}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if out is not None:
        write_detail(args, detail)
        print(json.dumps(out), flush=True)


def write_detail(args, detail: dict) -> None:
    """Per-stage timings, autotuner candidates and the legs' full records
    (bench_detail.json); the JSON line keeps the headline figures."""
    d = args.detail_dir or "."
    try:
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "bench_detail.json"), "w") as f:
            json.dump(detail, f, indent=1)
    except OSError:
        pass


def default_wave_paths(pixels: int) -> int:
    """The library's default paths per wave set (default_wave_paths in
    cudart_gb300/csrc/crt_internal.h)."""
    cap = 1 << 16
    while cap < pixels * 16 and cap < (1 << 25):
        cap <<= 1
    return cap


def run_build_only(args) -> None:
    """Scene creation alone (host arrays -> device scene with its BVH), the
    part of the end-to-end step before rendering; one JSON line."""
    import torch
    from cudart_gb300 import GB300Scene, scenes
    sc = scenes.large_textured() if not args.small else scenes.large_textured(
        width=480, height=270, grid=256, tex_size=256)
    wall, build = [], []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = GB300Scene(sc, builder=args.build_only)
        torch.cuda.synchronize()
        if k >= args.warmup:
            wall.append(time.perf_counter() - t0)
            build.append(s.info.build_ms)
        info = s.info
        del s
    print(json.dumps({"metric": "scene_create_ms", "builder": args.build_only, "triangles": sc.n_tris,
                      "nodes": int(info.num_nodes), "max_depth": int(info.max_depth),
                      "wall_ms": round(1e3 * statistics.median(wall), 2),
                      "build_ms": round(statistics.median(build), 2), "steps": args.steps}))


def _ref_load_once(obj: str, cam: str, tex: str, w: int, h: int) -> float:
    """The reference's own loader (Scene::loadObj, loadCamera, loadTextures,
    loadTriangles; oracle/_ref, built where the CudaRT sources are) in ms."""
    import ctypes as C
    L = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcrt_ref.so"))
    L.ref_time_load.restype = C.c_double
    L.ref_time_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int]
    return float(L.ref_time_load(obj.encode(), cam.encode(), tex.encode(), w, h))


def run_ingest(args) -> None:
    """Scene-file loading on the host: crt_scene_files_load +
    crt_camera_load_json on the OBJ/MTL/JSON/PNG files of a workload (best of
    --steps), beside the reference's loader on the same files as the CPU
    baseline when oracle/_ref exists (one load, in a process of its own: the
    reference keeps loader state in static variables).  One JSON line."""
    from cudart_gb300 import SceneFiles, load_camera_json, scenes
    sc = getattr(scenes, args.ingest)()
    with tempfile.TemporaryDirectory() as td:
        files = scenes.write_reference_files(sc, td, args.ingest)
        obj_bytes = os.path.getsize(files["obj"])
        lib_ms, parse_ms = [], []
        for _ in range(max(1, args.steps)):
            t = time.perf_counter()
            f = SceneFiles(files["obj"], files["textures"])
            load_camera_json(files["camera"], sc.width, sc.height)
            lib_ms.append((time.perf_counter() - t) * 1e3)
            parse_ms.append(float(f.info.parse_ms))
            assert f.n_tris == sc.n_tris
            f.close()
        ref_ms = None
        if os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libcrt_ref.so")):
            p = subprocess.run([sys.executable, os.path.abspath(__file__), "--ref-load-once", files["obj"],
                                files["camera"], files["textures"], str(sc.width), str(sc.height)],
                               capture_output=True, text=True, check=True)
            ref_ms = float(p.stdout.strip().splitlines()[-1])
    best = min(lib_ms)
    print(json.dumps({"metric": "scene_files_load_ms", "scene": args.ingest, "triangles": sc.n_tris,
                      "obj_mb": round(obj_bytes / 1e6, 1), "library_ms": round(best, 1),
                      "library_parse_ms": round(min(parse_ms), 1),
                      "library_mb_per_s": round(obj_bytes / 1e3 / best, 1),
                      "cpu_baseline": None if ref_ms is None else {
                          "value": round(ref_ms, 1), "unit": "ms", "kind": "reference", "cores": 1,
                          "sample": "Scene::loadObj + loadCamera + loadTextures + loadTriangles, one load"},
                      "speedup": None if ref_ms is None else round(ref_ms / best, 1),
                      "host_threads": os.cpu_count()}), flush=True)


def main():
    if len(sys.argv) == 7 and sys.argv[1] == "--ref-load-once":
        obj, cam, tex, w, h = sys.argv[2:]
        print(_ref_load_once(obj, cam, tex, int(w), int(h)))
        return
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--spp", type=int, default=256)
    ap.add_argument("--small", action="store_true", help="480x270 reduced scene (profiling)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true", help="default launch options, no autotuner")
    ap.add_argument("--options", default="", help='with --no-tune: launch options as JSON, e.g. {"node_format": "f32"}')
    ap.add_argument("--no-extra", action="store_true", help="skip the batched-views and adjoint legs")
    ap.add_argument("--c4-spp-div", type=int, default=1,
                    help="batched views: spp divisor (1 = the workload's own spp)")
    ap.add_argument("--detail-dir", default="", help="directory for bench_detail.json")
    ap.add_argument("--inversion-iters", type=int, default=200)
    ap.add_argument("--inversion-loss", default="clamped", choices=["clamped", "masked", "hdr"])
    ap.add_argument("--inversion-study", action="store_true",
                    help="run the material-inversion variants (loss, roulette mode) and exit")
    ap.add_argument("--ingest", default=None, choices=["mixed_mid", "large_textured"],
                    help="time scene-file loading of this workload on the host and exit")
    ap.add_argument("--build-only", choices=["gpu", "host"], default=None,
                    help="time crt_scene_create with this BVH builder on the 1080p scene and exit")
    args = ap.parse_args()
    if args.ingest:
        run_ingest(args)
    elif args.build_only:
        run_build_only(args)
    elif args.inversion_study:
        inversion_study(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
