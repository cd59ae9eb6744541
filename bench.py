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
  node and triangle fetches counted by an untimed re-run) against the
  measured HBM copy bandwidth.
* cpu_baseline / --impl reference: the CPU oracle port of the reference's
  `--cpu` path on all host threads over a bounded pixel sample.

Under torchrun each rank renders its own sample range of the same frame
(weak scaling, no collective on the data path).
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
        b.render()
        e.record(stream)
        torch.cuda.synchronize()
        ms = s.elapsed_time(e)
        res[name] = {"ms": round(ms, 2), "msamples_per_s": round(samples / (ms * 1e-3) / 1e6, 2)}
        del b
    plain = max(("sequential_plain_q8", "sequential_plain_f32"), key=lambda k: res[k]["msamples_per_s"])
    res["sequential_plain"] = dict(res[plain], node_format=plain.rsplit("_", 1)[1])
    out.update(res)
    out["speedup"] = round(res["batched_wavefront"]["msamples_per_s"] / res["sequential_plain"]["msamples_per_s"], 3)
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
    # inversion
    kd = kd_true.copy()
    kd[boxes] = 0.5
    m1 = np.zeros_like(kd)
    m2 = np.zeros_like(kd)
    b1, b2, lr, eps = 0.9, 0.999, 1e-2, 1e-8
    err0 = float(np.sqrt(np.mean((kd[boxes] - kd_true[boxes]) ** 2)))

    def image_loss(kd_vals):
        """L2 image loss of a 1024-spp render (its own sample range) against
        the target: the optimisation's progress without the noise of one
        64-spp iteration."""
        g.set_materials(kd=kd_vals)
        r.restart(1 << 25)   # not the target's samples (1 << 24) nor the iterations'
        r.render(1024)
        img = torch.from_numpy(r.accum()).cuda() / 1024
        return float(((img.clamp(0, 1) - target.clamp(0, 1)) ** 2).sum())

    clean0 = image_loss(kd)
    losses = []
    t0 = time.perf_counter()
    for it in range(args.inversion_iters):
        g.set_materials(kd=kd)
        r.restart(it * sc.spp)
        r.render(sc.spp)
        img = torch.from_numpy(r.accum()).cuda() / sc.spp
        # L2 on display-range radiance (clamped to [0, 1], as the RGBA8 output
        # quantises it): the unbounded HDR loss is dominated by a few
        # fireflies near the lights
        diff = img.clamp(0, 1) - target.clamp(0, 1)
        loss = float((diff ** 2).sum())
        losses.append(loss)
        adj[:, :3] = 2.0 * diff * (img < 1).float() / sc.spp
        gkd.zero_()
        gka.zero_()
        r.adjoint((1 << 23) + it * sc.spp, sc.spp, adj.data_ptr(), gkd.data_ptr(), gka.data_ptr())
        r.synchronize()
        grad = gkd.cpu().numpy()
        grad[np.setdiff1d(np.arange(n_mats), boxes)] = 0.0
        m1 = b1 * m1 + (1 - b1) * grad
        m2 = b2 * m2 + (1 - b2) * grad * grad
        step = lr * (m1 / (1 - b1 ** (it + 1))) / (np.sqrt(m2 / (1 - b2 ** (it + 1))) + eps)
        kd = np.clip(kd - step, 0.01, 0.99).astype(np.float32)
        if it == 0:
            loss0 = loss
    seconds = round(time.perf_counter() - t0, 2)
    clean1 = image_loss(kd)
    g.set_materials(kd=kd_true)
    q = max(1, min(20, len(losses) // 4))
    out["inversion"] = {"iterations": args.inversion_iters, "lr": lr, "loss_first": round(loss0, 4),
                        "loss_last": round(loss, 4),
                        "loss_median_first_iters": round(float(np.median(losses[:q])), 4),
                        "loss_median_last_iters": round(float(np.median(losses[-q:])), 4),
                        "image_loss_1024spp_start": round(clean0, 4),
                        "image_loss_1024spp_end": round(clean1, 4),
                        "albedo_rmse_start": round(err0, 4),
                        "albedo_rmse_end": round(float(np.sqrt(np.mean((kd[boxes] - kd_true[boxes]) ** 2))), 4),
                        "seconds": seconds,
                        "note": "loss_first / loss_last are single noisy 64-spp iterations; the medians and "
                                "the 1024-spp image losses (own samples) are the noise-robust measures"}
    return out


def run_gb300(args):
    import numpy as np
    import torch
    from cudart_gb300 import GB300Renderer, GB300Scene, autotune, options_dict, scenes

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
        tune = autotune(scene, sc.width, sc.height, max_depth=sc.max_depth, trial_spp=32, repeats=2,
                        rounds=1, tune_bvh_width=False)
        tuned = {"options": {k: v for k, v in options_dict(tune.options).items()
                             if k not in ("seed", "max_depth", "view_id")},
                 "candidates": tune.candidates, "seconds": round(time.perf_counter() - t0, 2),
                 "start_ms_per_spp": round(tune.start_ms_per_spp, 3),
                 "tuned_ms_per_spp": round(tune.ms_per_spp, 3)}
        opts = tune.options
        opts.seed, opts.view_id = 1234, rank
        wf = GB300Renderer(scene, sc.width, sc.height, spp, options=opts)
    else:
        # each rank renders its own Philox streams of the same frame (view_id = rank);
        # --options sets launch options by hand (e.g. to profile one variant)
        extra = json.loads(args.options) if args.options else {}
        wf = GB300Renderer(scene, sc.width, sc.height, spp, max_depth=sc.max_depth, seed=1234,
                           mode="wavefront", view_id=rank, **extra)
    wf.set_stream(stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed_steps(r, k_steps):
        durs = []
        for k in range(k_steps):
            flush.fill_(float(k))
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            r.reset()
            s.record(stream)
            r.render(spp)
            e.record(stream)
            durs.append((s, e))
        torch.cuda.synchronize()
        return [s.elapsed_time(e) for s, e in durs]

    for _ in range(args.warmup):
        wf.reset()
        wf.render(spp)
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
                           mode="megakernel", view_id=rank, node_format=fmt)
        mk.set_stream(stream.cuda_stream)
        mk.reset()
        mk.render(spp)
        torch.cuda.synchronize()
        plain_by_format[fmt] = sum(timed_steps(mk, k_plain)) / k_plain
        identical = identical and bool(np.array_equal(mk.accum(), wf_acc))
        del mk
    plain_fmt = min(plain_by_format, key=plain_by_format.get)
    mk_ms = plain_by_format[plain_fmt]
    plain_value = npix * spp / (mk_ms * 1e-3) / 1e6

    out = None
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
        for stage, rays, nodes, tris in (("extend", "extension_rays", "extension_nodes", "extension_tris"),
                                         ("shadow", "shadow_rays", "shadow_nodes", "shadow_tris")):
            launches = prof[f"{stage}_launches"]
            alg = prof[nodes] * node_bytes + prof[tris] * TRI_BYTES
            ms_l = prof[f"{stage}_ms"] / launches
            gbs = alg / launches / (ms_l * 1e-3) / 1e9
            roof[stage] = {"kernel": "wf_" + stage, "bytes_per_launch": alg / launches,
                           "ms_per_launch": ms_l, "gbs": gbs, "rays": prof[rays],
                           "nodes_per_ray": prof[nodes] / max(prof[rays], 1),
                           "tris_per_ray": prof[tris] / max(prof[rays], 1)}
        main = roof["extend"] if dom != "shadow" else roof["shadow"]
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic_per_ray.json")
        if os.path.exists(tp):
            fmt = "f32" if wf.options.node_format == 1 else "q8"
            tr = json.load(open(tp)).get(main["kernel"], {}).get(fmt)
            if tr:
                traffic = round(tr["dram_bytes_per_ray"] * main["rays"] / prof[f"{dom if dom in roof else 'extend'}_launches"])
        roofline = {"bound": "hbm", "kernel": main["kernel"], "achieved": round(main["gbs"], 1),
                    "peak": peak, "unit": "GB/s", "frac": round(main["gbs"] / peak, 4),
                    "traffic": traffic, "peak_kind": f"{peak_kind} (HBM copy)",
                    "algorithmic_bytes": f"nodes visited x {node_bytes} B + triangles tested x 48 B per ray",
                    "dram_share_of_algorithmic": (round(traffic / main["bytes_per_launch"], 4)
                                                  if traffic else None),
                    "reading": "achieved counts the node and triangle bytes the traversal consumes; most are "
                               "L1/L2 hits (traffic is the DRAM part), so frac can exceed 1: the kernel is "
                               "issue/latency-bound, not HBM-bound",
                    "stage_ms": {s: round(prof[f"{s}_ms"], 2) for s in stages},
                    "profile_spp": 8,
                    "extend_rays_by_bounce": prof["extend_rays_by_bounce"][:sc.max_depth],
                    "extend_ms_by_bounce": [round(x, 3) for x in prof["extend_ms_by_bounce"][:sc.max_depth]],
                    "stages": {k: {kk: (round(vv, 3) if isinstance(vv, float) else vv)
                                   for kk, vv in v.items()} for k, v in roof.items()}}
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
        out = {
            "metric": METRIC, "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator: heightfield value noise, procedural texture)",
            "config": {"workload": WORKLOAD, "mode": "wavefront (CUDA-graph waves, concurrent wave sets)",
                       "width": sc.width, "height": sc.height, "spp": spp, "max_depth": sc.max_depth,
                       "triangles": info.num_triangles, "bvh_nodes": info.num_nodes,
                       "bvh_depth": info.max_depth, "autotune": tuned,
                       "l2": "flushed before every step (256 MiB write); scene buffers > L2"},
            "plain_kernel": {"value": round(plain_value, 3), "ms_per_step": round(mk_ms, 3),
                             "node_format": plain_fmt,
                             "ms_per_step_by_node_format": {k: round(v, 3) for k, v in plain_by_format.items()},
                             "accum_identical_to_wavefront": identical},
            "speedup_vs_plain": round(value / world / plain_value, 3),
            "mrays_per_s": round(value * rays_per_sample, 1),
            "rays_per_sample": round(rays_per_sample, 3),
            "adjoint_forward_ratio": c5["ratio"] if c5 else None,
            "batched_views": c4, "adjoint": c5,
            "clocks": clocks, "gpu_launches": launches, "e2e": e2e, "roofline": roofline,
            "cpu_baseline": cpu,
        }
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


def default_wave_paths(pixels: int) -> int:
    """The library's default paths per wave set (default_wave_paths in
    cudart_gb300/csrc/crt_internal.h)."""
    cap = 1 << 16
    while cap < pixels * 8 and cap < (1 << 24):
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


def main():
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
    ap.add_argument("--c4-spp-div", type=int, default=4, help="batched views: spp divisor")
    ap.add_argument("--inversion-iters", type=int, default=200)
    ap.add_argument("--build-only", choices=["gpu", "host"], default=None,
                    help="time crt_scene_create with this BVH builder on the 1080p scene and exit")
    args = ap.parse_args()
    if args.build_only:
        run_build_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
