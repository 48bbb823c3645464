"""DRMLT hot-path benchmark: mutations/s of the GPU chain loop on one GB300.

Workload (default): the H2MC second-stage configuration -- the Phong Cornell
box (34 + 2 triangles) at 1024x1024, max depth 8, 16384 chains, type=mira,
stage-2 anisotropic probability 0.5, sigma 1/64 -- written by
drmlt/scenegen.py:config2 from a fixed seed (synthetic scene; the reference
publishes no benchmark scene). One step = one DR iteration of every chain
(16384 mutations). `value` is device-timed mutations/s over K steps with the
chain state resident in HBM; `e2e` is the same metric through the public C ABI
from host buffers (scene upload, prepass, direct pass, K steps, film readback).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload config2|config4|config5]

--workload config4 / config5 run the large procedural scenes of
drmlt/procedural.py instead (3.0 M / 8.0 M triangles, max depth 12, 65536 /
262144 chains; scene built in memory). Their CPU legs are not run: the
oracle's brute-force intersector costs O(triangles) per ray.

Under torchrun (N > 1) every rank renders its own shard of chains (different
random streams) and the films are summed; chains are independent, so there is
no collective in the timed region.
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
WORKLOAD = "drmlt-h2mc-phong-cornell-1024x1024-depth8-16384chains-mira"
METRIC = "mutations_per_second"


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


def write_workload(tmp: str, spp: int = 64) -> str:
    from drmlt import scenegen
    return scenegen.write_cornell(os.path.join(tmp, "cfg2"), seed=2, width=1024, height=1024, phong=True,
                                  options=scenegen.SceneOptions(maxdepth=8, numchains=16384, spp=spp, type="mira"))


LARGE = {
    "config4": ("drmlt-h2mc-displaced-sphere-3.0Mtris-env-point-1024x1024-depth12-65536chains-mira", "config4"),
    "config5": ("drmlt-h2mc-caustic-heightfield-8.0Mtris-2048x2048-depth12-262144chains-mira", "config5"),
}


def load_workload(name: str, tmp: str):
    """(scene data, XML path or None, workload label) of a bench workload."""
    from drmlt import procedural
    from drmlt import scene as dscene
    if name == "config2":
        xml = write_workload(tmp)
        return dscene.load_scene(xml), xml, WORKLOAD
    label, fn = LARGE[name]
    # enough samples per pixel that the autotuner, warm-up and timed steps fit in one render
    return getattr(procedural, fn)(spp=128 if name == "config4" else 32), None, label


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of each chain-loop
# kernel per iteration (both chain groups), from `ncu --set full` captures of
# the same kernels on these workloads; None where not captured.
NCU_TRAFFIC = {
    "config2": {"stage1": 2 * 3.47e6, "derivs_x": 2 * 0.63e6, "gauss_x": 2 * 0.82e6, "stage2": 2 * 2.00e6,
                "derivs_z": 2 * 0.67e6, "gauss_z": 2 * 2.29e6, "finish": 2 * 5.34e6},
    "config4": {"stage1": 2 * 145.7e6},
}

# Floating-point operations (FP32, FP64) of the derivative and Gaussian
# kernels per chain-loop iteration (both chain groups): ncu's executed-op
# counters (smsp__sass_thread_inst_executed_op_{fadd,fmul,ffma}_pred_on.sum and
# the d-variants, an FMA counted as 2) summed over the bench's own launches of
# these kernels after the autotuner; None where not captured.
NCU_FLOPS = {
    "config2": {"derivs_x": (7.256e8, 0.0), "derivs_z": (7.500e8, 0.0),
                "gauss_x": (9.821e7, 2.690e7), "gauss_z": (1.059e8, 4.613e7)},
}

# Algorithmic bytes each stage moves per chain (read + write of chain state in
# HBM). A Slot is 328 B, the per-chain scratch 128 B (both asserted in
# csrc/chain.cuh), a stored FP64 Gaussian 5008 B.
SLOT_B = 328
SCRATCH_B = 128
GAUSS_B = 8 * (24 * 24 + 2 * 24 + 2)


def run_ours(args, world, rank, local):
    import torch
    from drmlt import scene as dscene
    from drmlt.integrator import Renderer

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp()
    sd, xml, label = load_workload(args.workload, tmp)
    N = sd.options.numChains
    seed = 0x1234ABCD + 7919 * rank

    # ---- device-timed throughput (chain state resident in HBM)
    r = Renderer(sd, device=local, seed=seed)
    r.direct()
    r.prepass()
    lanes, dwarps = r.autotune(8)  # launch shape for this scene (drmlt_autotune)
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
    rays = ray_roofline(r, _peaks()[0]) if rank == 0 else None
    fma = {"fp32_tflops": r.fma_benchmark(False)["tflops"], "fp64_tflops": r.fma_benchmark(True)["tflops"]} \
        if rank == 0 else None
    r.close()
    dev_ms, done_all = replica_totals(dev_ms, done, world, "cuda")
    value = done_all / (dev_ms * 1e-3)

    # ---- end to end through the C ABI: host scene -> film on the host (scene
    # upload, bootstrap prepass, K steps, film readback; the direct-lighting pass
    # is not part of the mutation metric and is left out on both arms)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    r2 = Renderer(sd, device=local, seed=seed + 1)
    r2.prepass()
    r2.autotune(8)
    r2.run(args.steps)
    film = r2.film()
    e2e_s = time.perf_counter() - t0
    e_done = r2.stats()["mutations"]  # the autotuner's iterations included
    r2.close()
    scene_bytes = sd.positions.nbytes + sd.normals.nbytes + 64 * 4
    e2e = {"value": e_done / e2e_s * world, "unit": "mutations/s", "h2d_bytes_per_step": scene_bytes // args.steps,
           "d2h_bytes_per_step": film.nbytes // args.steps}

    # ---- roofline of the dominant stage kernel
    hbm, peak_kind = _peaks()
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
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": NCU_TRAFFIC.get(args.workload, {}).get(dom), "peak_kind": peak_kind,
            "stage_ms_per_iteration": {k: v / iters for k, v in prof.items()}}

    # ---- compute rooflines: derivative kernel on the FP32 FMA roof, Gaussian
    # kernel on the FP64 roof, both against this device's measured FMA peaks
    compute = None
    if fma is not None:
        compute = {"peaks_measured": fma}
        for st in ("derivs_x", "derivs_z", "gauss_x", "gauss_z"):
            ms = prof[st] / iters
            ent = {"ms_per_iteration": ms}
            counts = NCU_FLOPS.get(args.workload, {}).get(st)
            if counts is not None:
                for kind, n, peak in (("fp32", counts[0], fma["fp32_tflops"]), ("fp64", counts[1], fma["fp64_tflops"])):
                    a = n / (ms * 1e-3) / 1e12
                    ent[kind] = {"flops_per_iteration": n, "achieved": a, "peak": peak, "unit": "TFLOP/s",
                                 "frac": a / peak}
            compute[st] = ent

    out = None
    if rank == 0:
        relmse = relmse_plain = None
        if not args.no_relmse:
            ref_spp = args.ref_spp
            ref = render_reference(sd, local, ref_spp)
            spp = args.relmse_spp or (64 if args.workload == "config2" else 128)
            relmse = time_to_relmse(sd, local, ref, ref_spp, spp=spp)
            relmse_plain = time_to_relmse(sd, local, ref, ref_spp, spp=spp, plain=True)
        if xml is None:
            cpu = {"value": None, "unit": "mutations/s", "cores": 0, "kind": "port",
                   "sample": "not run: the oracle's brute-force intersector costs O(triangles) per ray"}
        else:
            cpu = cpu_baseline_sample(xml) if not args.no_cpu else None
        gb = (3 * SLOT_B + 3 * GAUSS_B + SCRATCH_B) * N / 1e9
        out = {
            "metric": METRIC, "value": value, "unit": "mutations/s", "n_gpus": world, "steps": args.steps,
            "steps_done": round(done / N),  # fewer than steps when the render ran out of iterations
            "warmup": args.warmup, "ms_per_step": dev_ms / max(1, round(done / N)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": label, "chains": N, "width": sd.width, "height": sd.height,
                       "max_depth": sd.options.maxDepth, "triangles": int(len(sd.positions)),
                       "dr_type": sd.options.type, "mutations_per_step": N * world,
                       "launch_shape": dict(shape, autotuned=True),
                       "l2": "chain state (3 slots + 3 FP64 Gaussians per chain, %.2f GB) exceeds L2" % gb},
            "e2e": e2e,
            "roofline": roof,
            "compute_roofline": compute,
            "cpu_baseline": cpu,
            "rays": rays,
            "time_to_relmse": relmse,
            "time_to_relmse_plain": relmse_plain,
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


def ray_roofline(r, hbm_gbs, n_rays=1 << 21, repeats=10):
    """Rays/s of the BVH traversal kernel alone on the workload's scene
    (drmlt_ray_benchmark) and the bytes it visits: nodes fetched x 64 B +
    triangles tested x 48 B per pass over the kernel's event-timed duration,
    against the HBM peak (the upper levels of the tree sit in L2, so the
    fraction can exceed what DRAM alone delivers)."""
    out = {}
    for kind in r.RAY_KINDS:
        b = r.ray_benchmark(kind, n_rays, repeats)
        sec = b["ms"] * 1e-3
        gbs = (64.0 * b["nodes"] + 48.0 * b["tris"]) / sec / 1e9
        out[kind] = {"rays_per_s": b["rays"] / sec, "ms_per_pass": b["ms"], "rays": int(b["rays"]),
                     "nodes_per_ray": b["nodes"] / max(b["rays"], 1), "tris_per_ray": b["tris"] / max(b["rays"], 1),
                     "visited_gbs": gbs, "frac_of_hbm": gbs / hbm_gbs}
    return out


def rel_mse(img, ref):
    """Mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2)."""
    return float(np.mean((img - ref) ** 2 / (ref * ref + 1e-2)))


# The plain per-stage-launch GPU drop-in: the same kernels launched one stage
# at a time on one stream without CUDA graphs, one chain per lane in the
# per-chain kernels, one warp per chain's derivatives, no launch autotuning.
PLAIN = dict(use_graph=0, chain_groups=1, stage_lanes=32, stage2_lanes=32, deriv_warps=1)


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


def time_to_relmse(sd, device, ref, ref_spp, target=0.01, spp=None, plain=False):
    """Seconds of GPU rendering until the image is within relMSE `target` of a
    long render (`ref`, ref_spp samples per pixel, other random streams) of the
    same scene: the direct-lighting pass, the prepass (and the autotuner's
    iterations) plus the chain-loop device time up to the first checkpoint
    that meets the target (iteration counts growing by 1.25x, by 1/32 once the
    relMSE is within 1.5x of the target, so the crossing is resolved to ~3%).
    Partial images scale the indirect film by total / done iterations.
    plain=True runs the plain per-stage-launch configuration (PLAIN) without
    autotuning."""
    from drmlt.integrator import Renderer

    kw = dict(PLAIN) if plain else {}
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
    r.close()
    return {"value": hit, "unit": "s", "target_relmse": target, "reference": "%d spp GPU render, direct pass at %d spp" % (ref_spp, 64 * max(1, sd.options.directSpp)),
            "setup_s": setup_s, "iterations": done, "spp_equivalent": done * sd.options.numChains /
            (sd.width * sd.height), "mutations_per_s": done * sd.options.numChains / max(run_s, 1e-9),
            "checkpoints": checkpoints}


def cpu_baseline_sample(xml: str, seconds: float = 15.0):
    """The oracle's CPU restatement of the chain loop on this host's cores, on a
    bounded sample of the same workload."""
    try:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle_dr  # noqa: WPS433
    except Exception as e:  # oracle not built on this machine
        return {"value": None, "unit": "mutations/s", "cores": 0, "kind": "port", "sample": "unavailable: %s" % e}
    return oracle_dr.cpu_throughput(xml, seconds=seconds)


def run_reference(args, world, rank):
    """Reference arm: the reference's CPU algorithm (oracle restatement, all host
    cores) on the same workload, metric and unit."""
    if rank != 0:
        return None
    tmp = tempfile.mkdtemp()
    xml = write_workload(tmp)
    try:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle_dr
    except Exception as e:
        return {"impl": "reference", "unavailable": "oracle CPU port not built: %s" % e}
    per = min(15.0, max(0.25, 90.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        oracle_dr.cpu_throughput(xml, seconds=per)
    vals = [oracle_dr.cpu_throughput(xml, seconds=per) for _ in range(args.steps)]
    v = statistics.median([x["value"] for x in vals])
    cpu = dict(vals[0])
    cpu["value"] = v
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "mutations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD}, "cpu_baseline": cpu,
            "e2e": {"value": v, "unit": "mutations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-relmse", action="store_true", help="skip the time-to-relMSE measurement")
    ap.add_argument("--workload", default="config2", choices=["config2", "config4", "config5"])
    ap.add_argument("--ref-spp", type=int, default=256, help="samples per pixel of the relMSE reference render")
    ap.add_argument("--relmse-spp", type=int, default=0, help="spp budget of the time-to-relMSE renders")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_ours(args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
