"""DRMLT hot-path benchmark: mutations/s and time to relMSE 0.01 of the GPU
chain loop on one GB300.

Workload (default ``config4``): the batched persistent-DRMLT configuration --
a displaced geodesic sphere of 1,997,120 triangles (rough dielectric) over a
Phong ground grid of 1,002,528 triangles, a constant environment map and a
point light, 1024x1024, max depth 12, 65536 chains, type=mira, built in memory
by drmlt/procedural.py:config4 from a fixed seed (synthetic scene: the
reference publishes no benchmark scene). One step = one DR iteration of every
chain (65536 mutations).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload config4|config2|config5]

Keys of the JSON line (ours):
  value            device-timed mutations/s over K graph-launched steps, chain
                   state resident in HBM (1.06 GB, larger than L2)
  e2e              the same metric through the C ABI as a user calls it: K
                   steps, each drmlt_run_async(1) with a copy of the statistics
                   into pinned host memory and a host read of the previous
                   step's statistics (drmlt_wait_stats: one step in flight),
                   then the film read back; the one-time set-up
                   (scene upload from host buffers, BVH build, prepass) is
                   timed separately (setup_s) and given with it as
                   value_with_setup
  time_to_relmse   seconds (direct pass, prepass, autotuning, chain loop) until
  (_plain,         relMSE <= 0.01 against a long render, for the batched form
   _adjoint)       (hyper-dual derivatives), the plain per-stage-launch drop-in
                   and the batched form with the reverse-mode adjoint taking
                   the derivatives of paths of dimension 10 and up
  roofline         the slowest chain-loop stage against the HBM peak
  cpu_baseline     the oracle's CPU chain loop (all host cores, the oracle's
                   own BVH) on a bounded sample of the same scene, with its
                   calibration against the reference's own dpt chain loop
  schedule_ms_per_iteration
                   the staged (default), wavefront and persistent schedules of
                   the same steps, a few iterations each

--impl reference times that CPU chain loop alone on the same workload (the
reference's sources, from which its dpt is built, are not on the GPU host; the
calibration factor relates the two). Under torchrun (N > 1) every rank renders its own
replica of the chains (different random streams); there is no collective in
the timed region, and --gpus must equal the torchrun world size.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "drmlt-dpt_gb300"))

import numpy as np  # noqa: E402

PEAKS_PATH = os.path.join(REPO, "MEASURED_PEAKS.json")
COUNTERS_PATH = os.path.join(REPO, "profiles", "ncu_counters.json")
METRIC = "mutations_per_second"
L2_BYTES = 129e6


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_totals(dev_ms: float, done: int, world: int, device: str = "cpu"):
    """Independent replicas (one per rank, no data exchange): the slowest rank's
    timed-region device time and the mutations of all ranks."""
    if world <= 1:
        return dev_ms, done
    import torch
    import torch.distributed as dist
    t = torch.tensor([dev_ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(done)], device=device, dtype=torch.float64)
    dist.all_reduce(n)
    return float(t.item()), int(n.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# workload -> (label, relMSE reference spp, time-to-relMSE spp budget)
WORKLOADS = {
    "config4": ("drmlt-h2mc-displaced-sphere-3.0Mtris-env-point-1024x1024-depth12-65536chains-mira", 512, 128),
    "config2": ("drmlt-h2mc-phong-cornell-1024x1024-depth8-16384chains-mira", 256, 64),
    "config5": ("drmlt-h2mc-caustic-heightfield-8.0Mtris-2048x2048-depth12-262144chains-mira", 128, 32),
}
DEFAULT_WORKLOAD = "config4"


def load_workload(name: str, tmp: str):
    """(scene data, workload label) of a bench workload."""
    from drmlt import procedural
    from drmlt import scene as dscene
    from drmlt import scenegen
    label, _, spp = WORKLOADS[name]
    if name == "config2":
        xml = scenegen.write_cornell(os.path.join(tmp, "cfg2"), seed=2, width=1024, height=1024, phong=True,
                                     options=scenegen.SceneOptions(maxdepth=8, numchains=16384, spp=spp, type="mira"))
        return dscene.load_scene(xml), label
    # enough samples per pixel that the autotuner, warm-up and timed steps fit in one render
    return getattr(procedural, name)(spp=spp), label


def workload_config(sd, label: str) -> dict:
    """The `config` object both arms print for one workload."""
    return {"workload": label, "chains": int(sd.options.numChains), "width": int(sd.width), "height": int(sd.height),
            "max_depth": int(sd.options.maxDepth), "triangles": int(len(sd.positions)), "dr_type": sd.options.type}


def source_hash() -> str:
    """Hash of the CUDA/C++ sources and the ABI header: profiler counters are
    valid only for the build they were captured on."""
    import hashlib
    h = hashlib.sha256()
    csrc = os.path.join(REPO, "drmlt-dpt_gb300", "csrc")
    for f in sorted(os.listdir(csrc)) + ["../../include/drmlt_capi.h"]:
        with open(os.path.join(csrc, f), "rb") as fh:
            h.update(f.encode() + b"\0" + fh.read())
    return h.hexdigest()[:16]


def ncu_counters(workload: str):
    """DRAM bytes and FP32/FP64 flops per iteration of the chain-loop kernels
    from ncu captures (profiles/ncu_counters.json), when they were captured on
    this build's sources; else (None, reason)."""
    try:
        with open(COUNTERS_PATH) as f:
            c = json.load(f)
    except Exception as e:  # noqa: BLE001
        return None, "no counters file (%s)" % type(e).__name__
    mine = source_hash()
    if c.get("source_hash") != mine:
        return None, "captured on sources %s, this build is %s" % (c.get("source_hash"), mine)
    w = c.get("workloads", {}).get(workload)
    if w is None:
        return None, "no capture for %s" % workload
    return w, c.get("command")


# Algorithmic bytes each stage moves per chain (read + write of chain state in
# HBM). A Slot is 328 B, the per-chain scratch 128 B (both asserted in
# csrc/chain.cuh), a stored FP64 Gaussian 5008 B.
SLOT_B = 328
SCRATCH_B = 128
GAUSS_B = 8 * (24 * 24 + 2 * 24 + 2)


def run_ours(args, world, rank, local):
    import torch
    from drmlt.integrator import Renderer

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp()
    sd, label = load_workload(args.workload, tmp)
    N = sd.options.numChains
    seed = 0x1234ABCD + 7919 * rank

    # ---- device-timed throughput (chain state resident in HBM)
    r = Renderer(sd, device=local, seed=seed)
    r.direct()
    r.prepass()
    r.autotune(8)  # launch shape for this scene (drmlt_autotune)
    shape = r.launch_shape()
    r.run(args.warmup)
    prof, prof_mut = r.profile(max(1, min(8, args.steps)))  # per-stage CUDA-event times (serialised)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = r.kernel_launches()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        done = r.run(args.steps)
        wall = time.perf_counter() - t0
    launches = r.kernel_launches() - launches0
    dev_ms = r.last_run_ms()
    torch.cuda.synchronize()
    stats = r.stats()
    rays = ray_roofline(r, _peaks()[0], len(sd.positions)) if rank == 0 else None
    fma = {"fp32_tflops": r.fma_benchmark(False)["tflops"], "fp64_tflops": r.fma_benchmark(True)["tflops"]} \
        if rank == 0 else None
    r.close()
    dev_ms, done_all = replica_totals(dev_ms, done, world, "cuda")
    value = done_all / (dev_ms * 1e-3)

    # ---- end to end through the C ABI with host buffers, at the tuned launch
    # shape (no autotuning here): set-up = drmlt_create from the host scene
    # (upload + BVH build) and drmlt_prepass; then K steps, each enqueued with
    # its statistics copy (drmlt_run_async) before the host reads the previous
    # step's statistics (drmlt_wait_stats), and the film read back at the end
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    r2 = Renderer(sd, device=local, seed=seed + 1, autotune=0, stage_lanes=shape["chains_per_warp"],
                  stage2_lanes=shape["stage2_chains_per_warp"], deriv_warps=shape["derivative_warps"],
                  use_graph=1 if shape["graph_iterations"] else 0, graph_iters=max(1, shape["graph_iterations"]),
                  wavefront=shape["wavefront"], head_chains=shape["head_chains"], head_lanes=shape["head_lanes"],
                  adjoint_min_dim=shape["adjoint_min_dim"])
    r2.prepass()
    t1 = time.perf_counter()
    e_done = 0
    for k in range(args.steps):
        e_done += r2.run_async(1, k % 2)
        if k > 0:
            r2.wait_stats((k - 1) % 2)
    if args.steps > 0:
        r2.wait_stats((args.steps - 1) % 2)
    film = r2.film()
    t2 = time.perf_counter()
    r2.close()
    stats_bytes = 8 * 13  # the statistics counters copied per step
    scene_bytes = sd.positions.nbytes + sd.normals.nbytes
    e2e = {"value": e_done / (t2 - t1) * world, "unit": "mutations/s", "h2d_bytes_per_step": 0,
           "d2h_bytes_per_step": stats_bytes + film.nbytes // max(1, args.steps),
           "steps": args.steps, "mutations": e_done, "steps_s": t2 - t1, "setup_s": t1 - t0,
           "setup_h2d_bytes": scene_bytes,
           "value_with_setup": e_done / (t2 - t0) * world,
           "timed": "per step drmlt_run_async(1) (the step and a copy of its statistics into pinned host memory) "
                    "and drmlt_wait_stats of the previous step, drmlt_get_film at the end; set-up (drmlt_create "
                    "from host buffers incl. BVH build, drmlt_prepass) in setup_s"}

    # ---- roofline of the dominant stage kernel
    hbm, peak_kind = _peaks()
    counters, counters_src = ncu_counters(args.workload)
    stage_bytes = {
        "stage1": N * (2 * SLOT_B + SCRATCH_B),
        "stage2": N * (2 * SLOT_B + SCRATCH_B),
        "finish": N * (3 * SLOT_B + SCRATCH_B),
        "derivs_x": 0, "derivs_z": 0, "gauss_x": 0, "gauss_z": 0,
    }
    iters = max(1, prof_mut // N)
    dom = max(prof, key=prof.get)
    per_launch_ms = prof[dom] / iters
    # derivative / Gaussian stages: bytes = path records read + grad/Hessian or Gaussian written per listed chain
    if dom.startswith("derivs"):
        listed = max(1, stats["stage2_h2mc"] // max(1, stats["mutations"] // N)) if stats["mutations"] else 1
        stage_bytes[dom] = listed * (SLOT_B + 4 * (24 + 576))
    if dom.startswith("gauss"):
        listed = max(1, stats["stage2_h2mc"] // max(1, stats["mutations"] // N)) if stats["mutations"] else 1
        stage_bytes[dom] = listed * (4 * (24 + 576) + GAUSS_B)
    achieved = stage_bytes[dom] / (per_launch_ms * 1e-3) / 1e9
    traffic = counters.get("traffic", {}).get(dom) if counters else None
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
            "traffic_source": counters_src, "algorithmic_bytes_per_iteration": stage_bytes[dom],
            "stage_ms_per_iteration": {k: v / iters for k, v in prof.items()}}

    # ---- compute rooflines: derivative kernel on the FP32 FMA roof, Gaussian
    # kernel on the FP64 roof, both against this device's measured FMA peaks
    compute = None
    if fma is not None:
        compute = {"peaks_measured": fma, "flops_source": counters_src}
        for st in ("derivs_x", "derivs_z", "gauss_x", "gauss_z"):
            ms = prof[st] / iters
            ent = {"ms_per_iteration": ms}
            fl = counters.get("flops", {}).get(st) if counters else None
            if fl is not None:
                for kind, n, peak in (("fp32", fl[0], fma["fp32_tflops"]), ("fp64", fl[1], fma["fp64_tflops"])):
                    a = n / (ms * 1e-3) / 1e12
                    ent[kind] = {"flops_per_iteration": n, "achieved": a, "peak": peak, "unit": "TFLOP/s",
                                 "frac": a / peak}
            compute[st] = ent

    out = None
    if rank == 0:
        relmse = relmse_plain = relmse_adjoint = None
        if not args.no_relmse:
            _, ref_spp, budget = WORKLOADS[args.workload]
            ref_spp = args.ref_spp or ref_spp
            ref = render_reference(sd, local, ref_spp)
            spp = args.relmse_spp or budget
            relmse = time_to_relmse(sd, local, ref, ref_spp, spp=spp)
            relmse_plain = time_to_relmse(sd, local, ref, ref_spp, spp=spp, plain=True)
            # the batched form with the reverse-mode adjoint taking the H2MC
            # derivatives of paths of dimension 10 and up (drmlt_options.adjoint_min_dim)
            relmse_adjoint = time_to_relmse(sd, local, ref, ref_spp, spp=spp, extra=dict(adjoint_min_dim=10))
        cpu = None if args.no_cpu else cpu_baseline_sample(sd, seconds=15.0)
        schedules = None if args.no_schedules else schedule_times(sd, local, seed + 2, shape)
        gb = (3 * SLOT_B + 3 * GAUSS_B + SCRATCH_B) * N / 1e9
        out = {
            "metric": METRIC, "value": value, "unit": "mutations/s", "n_gpus": world, "steps": args.steps,
            "steps_done": round(done / N),  # fewer than steps when the render ran out of iterations
            "warmup": args.warmup, "ms_per_step": dev_ms / max(1, round(done / N)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": workload_config(sd, label),
            "mutations_per_step": N * world,
            "launch_shape": dict(shape, autotuned=True),
            "l2": "inputs larger than L2: chain state (3 slots + 3 FP64 Gaussians per chain, %.2f GB)%s" % (
                gb, ", BVH + triangles (%.0f MB)" % (len(sd.positions) * 124 / 1e6)
                if len(sd.positions) * 124 > L2_BYTES else ""),
            "e2e": e2e,
            "roofline": roof,
            "compute_roofline": compute,
            "cpu_baseline": cpu,
            "rays": rays,
            "time_to_relmse": relmse,
            "time_to_relmse_plain": relmse_plain,
            "time_to_relmse_adjoint": relmse_adjoint,
            "schedule_ms_per_iteration": schedules,
            "clocks": clk.summary(),
            "gpu_launches": launches,
            "wall_s_timed_region": wall,
            "acceptance": {k: stats[k + "_accepted"] / max(1, stats[k])
                           for k in ("large_step", "stage1", "stage2_iso", "stage2_h2mc")},
            "gaussians": {"anisotropic": stats["gaussians"], "fp64_jacobi_fallback": stats["gaussians_fp64_fallback"]},
        }
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def ray_roofline(r, hbm_gbs, n_tris, n_rays=1 << 21, repeats=10):
    """Rays/s of the BVH traversal kernel alone on the workload's scene
    (drmlt_ray_benchmark) and the bytes it visits (nodes fetched x 64 B +
    triangles tested x 48 B per pass over the kernel's event-timed duration).
    The bytes are quoted against the HBM peak only when the scene's BVH and
    triangles exceed L2; a smaller scene is cache-resident and its figure is
    given without an HBM fraction."""
    out = {}
    scene_bytes = n_tris * (48 + 36 + 36 + 4) + 32 * n_tris  # triangle records + ~n/2 64-byte nodes
    hbm_bound = scene_bytes > L2_BYTES
    for kind in r.RAY_KINDS:
        b = r.ray_benchmark(kind, n_rays, repeats)
        sec = b["ms"] * 1e-3
        gbs = (64.0 * b["nodes"] + 48.0 * b["tris"]) / sec / 1e9
        out[kind] = {"rays_per_s": b["rays"] / sec, "ms_per_pass": b["ms"], "rays": int(b["rays"]),
                     "nodes_per_ray": b["nodes"] / max(b["rays"], 1), "tris_per_ray": b["tris"] / max(b["rays"], 1),
                     "visited_gbs": gbs, "frac_of_hbm": gbs / hbm_gbs if hbm_bound else None}
    out["scene_bytes"] = scene_bytes
    out["residency"] = "HBM (scene larger than L2)" if hbm_bound else "L1/L2 (scene smaller than L2: no HBM fraction)"
    return out


def rel_mse(img, ref):
    """Mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2)."""
    return float(np.mean((img - ref) ** 2 / (ref * ref + 1e-2)))


# The plain per-stage-launch GPU drop-in: the chain loop's stages launched one
# at a time on one stream without CUDA graphs, one chain per lane tracing its
# whole path (no wavefront rounds), one warp per chain's derivatives by
# hyper-dual forward mode (no reverse-mode adjoint), no launch autotuning.
PLAIN = dict(use_graph=0, chain_groups=1, stage_lanes=32, stage2_lanes=32, deriv_warps=1, wavefront=0,
             adjoint_min_dim=-1)


def render_reference(sd, device, spp):
    """The relMSE reference: a long render of the same scene with other random
    streams, its direct-lighting pass also 64x longer than the scene's
    (at the scene's directspp the direct pass alone keeps two renders of
    config 4 ~0.005 apart in relMSE, whatever their chain budget)."""
    from drmlt.integrator import Renderer
    r = Renderer(sd, device=device, seed=0xBADC0FFE, spp=spp, direct_spp=64 * max(1, sd.options.directSpp))
    r.render()
    img = r.film().astype(np.float64)
    r.close()
    return img


def time_to_relmse(sd, device, ref, ref_spp, target=0.01, spp=None, plain=False, extra=None):
    """Seconds of GPU rendering until the image is within relMSE `target` of a
    long render (`ref`, ref_spp samples per pixel, other random streams) of the
    same scene: the direct-lighting pass, the prepass (and the autotuner's
    iterations) plus the chain-loop device time up to the first checkpoint
    that meets the target (iteration counts growing by 1.25x, by 1/32 once the
    relMSE is within 1.5x of the target, so the crossing is resolved to ~3%).
    Partial images scale the indirect film by total / done iterations.
    plain=True runs the plain per-stage-launch configuration (PLAIN) without
    autotuning; `extra` adds drmlt_options to the batched form."""
    from drmlt.integrator import Renderer

    kw = dict(PLAIN) if plain else dict(extra or {})
    if spp:
        kw["spp"] = spp
    r = Renderer(sd, device=device, seed=0x5EED1234, **kw)
    t0 = time.perf_counter()
    r.direct()
    r.prepass()
    direct_img = r.film().astype(np.float64)  # before any chain iteration: the direct pass alone
    if not plain:
        r.autotune(8)
    setup_s = time.perf_counter() - t0
    total = r.total_iterations()
    done = r.stats()["mutations"] // sd.options.numChains  # the autotuner's iterations (part of setup_s)
    run_s, hit, checkpoints = 0.0, None, []
    step = max(8, done)
    while done < total:
        n = min(step, total - done)
        r.run(n)
        run_s += r.last_run_ms() * 1e-3
        done += n
        img = direct_img + (r.film().astype(np.float64) - direct_img) * (total / done)
        e = rel_mse(img, ref)
        checkpoints.append([done, round(setup_s + run_s, 4), round(e, 6)])
        if e <= target:
            hit = setup_s + run_s
            break
        step = max(8, done // 4) if e > 1.5 * target else max(8, done // 32)
    shape = r.launch_shape()
    r.close()
    return {"value": hit, "unit": "s", "target_relmse": target, "launch_shape": shape, "reference": "%d spp GPU render, direct pass at %d spp" % (ref_spp, 64 * max(1, sd.options.directSpp)),
            "setup_s": setup_s, "iterations": done, "spp_equivalent": done * sd.options.numChains /
            (sd.width * sd.height), "mutations_per_s": done * sd.options.numChains / max(run_s, 1e-9),
            "checkpoints": checkpoints}


# The port against the reference's own chain loop on the same scene and
# threads, measured where the reference builds (x86, 8 threads, the config-2
# scene; oracle/ref/calibrate_cpu.py): the reference's dpt ran its chain loop
# at 0.416 M mutations/s (two renders differing only in spp, so prepass and
# direct pass cancel), the port at 0.181 M/s. The port is the slower of the
# two: CPU ratios against it overstate the GPU's lead by about 1 / 0.435.
CPU_CALIBRATION = {"port_over_reference": 0.435, "reference_mutations_per_s": 416343.0,
                   "port_mutations_per_s": 180926.0,
                   "measured": "x86_64, 8 threads, Phong Cornell box 1024x1024 depth 8 16384 chains mira; "
                               "reference dpt -d chain loop (spp 3 minus spp 1) vs the oracle port"}


def cpu_baseline_sample(sd, seconds: float = 15.0):
    """The oracle's CPU restatement of the chain loop (its own BVH) on this
    host's cores, on a bounded sample of the same workload."""
    try:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle_dr  # noqa: WPS433
    except Exception as e:  # oracle not built on this machine
        return {"value": None, "unit": "mutations/s", "cores": 0, "kind": "port", "sample": "unavailable: %s" % e}
    out = oracle_dr.cpu_throughput_scene(sd, seconds=seconds)
    out["calibration"] = CPU_CALIBRATION
    return out


def schedule_times(sd, device, seed, shape, iterations=8):
    """ms per iteration of the three chain-loop schedules (they take the same
    steps; the persistent one with hyper-dual derivatives throughout): staged at
    the tuned shape, wavefront rounds, and the persistent cooperative kernel (a
    quarter and half of the SMs as team workers)."""
    from drmlt.integrator import Renderer
    base = dict(autotune=0, stage_lanes=shape["chains_per_warp"], stage2_lanes=shape["stage2_chains_per_warp"],
                deriv_warps=shape["derivative_warps"], head_chains=shape["head_chains"], head_lanes=shape["head_lanes"],
                adjoint_min_dim=shape["adjoint_min_dim"])
    out = {}
    for name, kw in (("staged", {}), ("wavefront", dict(wavefront=1)), ("persistent_quarter", dict(persistent=1)),
                     ("persistent_half", dict(persistent=1, team_sms=76))):
        r = Renderer(sd, device=device, seed=seed, **base, **kw)
        r.prepass()
        r.run(4)
        r.run(iterations)
        out[name] = r.last_run_ms() / iterations
        r.close()
    return out


def run_reference(args, world, rank):
    """Reference arm: the reference's CPU algorithm (the oracle's restatement of
    the chain loop, all host cores, the oracle's own BVH) on the same workload,
    metric and unit. Each step is a bounded sample of the chain loop; the scene
    set-up and bootstrap prepass are outside the samples."""
    if rank != 0:
        return None
    tmp = tempfile.mkdtemp()
    sd, label = load_workload(args.workload, tmp)
    try:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle_dr
    except Exception as e:
        return {"impl": "reference", "unavailable": "oracle CPU port not built: %s" % e}
    loop = oracle_dr.CpuChainLoop(sd)
    per = min(15.0, max(0.5, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        loop.sample(per)
    vals = [loop.sample(per) for _ in range(args.steps)]
    loop.close()
    v = statistics.median([x["value"] for x in vals])
    cpu = dict(vals[0])
    cpu["value"] = v
    cpu["calibration"] = CPU_CALIBRATION
    cpu["sample"] = "median of %d samples of %.1f s: %s" % (len(vals), per, vals[0]["sample"])
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "mutations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(sd, label), "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "mutations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-relmse", action="store_true", help="skip the time-to-relMSE measurement")
    ap.add_argument("--no-schedules", action="store_true", help="skip the wavefront / persistent schedule timings")
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--ref-spp", type=int, default=0, help="samples per pixel of the relMSE reference render")
    ap.add_argument("--relmse-spp", type=int, default=0, help="spp budget of the time-to-relMSE renders")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.gpus != world:
        sys.exit("bench.py: --gpus %d but the torchrun world size is %d (launch N > 1 under torchrun)"
                 % (args.gpus, world))
    if args.warmup < 3:
        sys.exit("bench.py: at least 3 warm-up steps")
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
