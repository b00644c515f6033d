"""Benchmark: photon-transport throughput (histories/s) on the spiral-CT torso.

Workload (one step): 256x256x200 seeded six-material torso at 1.5 mm, spiral CT
120 kVp / 6 mm Al with the body bowtie, pitch 1.0, 40 mm collimation, 200 mm
scan, 360 exposures x 2,777,778 = 1.00e9 histories, Woodcock tracking against
the grid-wide majorant (--tracking macro|siddon for the other modes), FP64
scoring.  Inputs are seeded synthetic data of the configured shape (no
dataset exists for this path).

  value   histories/s over K timed steps with the world resident in HBM
  e2e     the same through the public C ABI with host buffers: H2D of the
          density/material arrays from pinned memory, World build, transport,
          D2H of the dose/variance/count arrays
  roofline  algorithmic bytes of the transport kernel (4 B per voxel visit, 48 B
          per deposit read-modify-write) / its CUDA-event time, vs measured HBM
  cpu_baseline  the CPU oracle (FP64 port of the path) on this host's cores, on a
          bounded sample of the same workload

`--impl reference` times that CPU implementation alone (the reference's own
engine, DXMClib, is fetched by its build at configure time and is not available).
N > 1 (torchrun): every rank runs its own full job on its own GPU with its own
random stream (independent histories; weak scaling, no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "s to \u22642% voxel dose error: MC+denoiser vs plain MC on 1 GB300; histories/s"
WORKLOAD = ("spiral CT on seeded synthetic torso 256x256x200 @1.5 mm (6 materials, +-2% density jitter), "
            "120 kVp 6 mm Al + body bowtie, pitch 1.0, 40 mm collimation, 200 mm scan, 1e9 histories")
# dram__bytes_read.sum + dram__bytes_write.sum per history, from 1-pass ncu captures of
# one 67,000,320-history transport launch of this workload (two regions on: 1.436 GB
# read + 0.799 GB written) and one 67,000,050-history launch of the 512x512x400
# workload (gather skip and two regions on: 10.96 GB + 2.80 GB).  The library's
# launches hold up to 2^28 histories; a launch's traffic is taken as these per-history
# figures times its histories (the tallies and voxels a launch touches grow with its
# histories).
TRAFFIC_BYTES_PER_HISTORY = 2.235e9 / 67_000_320
TRAFFIC_BYTES_PER_HISTORY_512 = 13.760e9 / 67_000_050
LAUNCH_HISTORIES = 1 << 28


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--histories", type=float, default=1e9, help="histories per step")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--tracking", choices=list(TRACKING), default="woodcock")
    p.add_argument("--macro-cell", type=int, default=16, help="macro-cell edge in voxels (macro tracking)")
    p.add_argument("--woodcock-steps", type=int, default=0,
                   help="Woodcock steps a lane takes between regroupings (0: library default)")
    p.add_argument("--gather-skip", type=int, choices=[-1, 0, 1], default=0,
                   help="Woodcock gather skip: 1 on, -1 off, 0 library default (on above 64 MiB of voxels)")
    p.add_argument("--two-region", type=int, choices=[-1, 0, 1], default=0,
                   help="two-region Woodcock (outside the box of non-air voxels against air's own majorant): "
                        "1 on, -1 off, 0 library default (on when the box of non-air voxels holds "
                        "less than half the grid)")
    p.add_argument("--interact-batch", type=int, default=0)
    p.add_argument("--refill-batch", type=int, default=0)
    p.add_argument("--correction", type=int, choices=[0, 1, 2], default=1,
                   help="bound-electron correction: 0 free electrons, 1 form factors (the reference's default), "
                        "2 impulse approximation + fluorescence")
    p.add_argument("--small", action="store_true", help="denoise-experiment: a small quick configuration")
    p.add_argument("--headline", choices=["full", "c5", "none"], default="full",
                   help="seconds to 2%% dose error, plain MC vs MC + denoiser, on the 512x512x400 spiral-CT "
                        "torso (c5), and also on a protocol the network was not trained on (full)")
    p.add_argument("--weights", default=str(ROOT / "opendxmc_gb300" / "weights" / "denoiser_torso_spiral.npy"),
                   help="trained denoiser parameters for the seconds-to-2%% measurement")
    p.add_argument("--conv-path", type=int, choices=[0, 1, 2], default=0,
                   help="denoiser: 0 default, 1 tcgen05 tensor cores, 2 mma.sync")
    p.add_argument("--inference-dims", default="512,512,400",
                   help="denoiser: x,y,z of the inference volume (multiples of 8)")
    p.add_argument("--save-weights", default="", help="denoise-experiment: write the trained parameters (.npy)")
    p.add_argument("--train-steps", type=int, default=0, help="denoise-experiment: training steps (0: default)")
    p.add_argument("--lr-final", type=float, default=0.0, help="denoise-experiment: final learning rate (0: default)")
    p.add_argument("--init-seeds", default="", help="denoise-experiment: initialisations to train, comma-separated; "
                   "the one best on a validation torso is kept (default: 0)")
    p.add_argument("--lows", default="", help="denoise-experiment: input history counts, comma-separated "
                   "(default 3e7,1e8,3e8,1e9)")
    p.add_argument("--workload", choices=["torso", "torso512", "c1", "batch", "pipelines", "denoiser",
                                          "world-denoise", "denoise-experiment", "c4-training"],
                   default="torso",
                   help="torso: the spiral-CT torso job (256x256x200); torso512: the 512x512x400 spiral-CT torso; "
                        "c1: the DX water cylinder (1e7 histories per step unless --histories); "
                        "batch: 64 uneven DX/CBCT jobs in one persistent launch; "
                        "pipelines: segmentation and organ dose table passes; denoiser: training step and "
                        "inference throughput; world-denoise: the world-path denoiser call on the 512x512x400 "
                        "torso after a 3e7-history run; c4-training: the denoiser trained on 200 seeded 128^3 "
                        "phantoms at 2 mm with 1e6/1e9-history pairs, scored on held-out phantoms")
    p.add_argument("--phantoms", type=int, default=200, help="c4-training: training phantoms")
    return p.parse_args()


TRACKING = {"woodcock": 0, "siddon": 1, "macro": 2}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


WORKLOAD_C1 = ("DX on a 128x128x64 water cylinder (16 cm, bone insert) at 1x1x2.5 mm, 70 kVp 2.5 mm Al, "
               "10x10 cm field at 100 cm, 1e7 histories")
WORKLOAD_512 = ("spiral CT on seeded synthetic torso 512x512x400 @0.8x0.8x1.0 mm (6 materials, +-2% density "
                "jitter), 120 kVp 6 mm Al + body bowtie, pitch 0.8, 80 mm collimation, 200 mm scan")


def workload(histories: float, big: bool = False, c1: bool = False, count_exposures=None):
    """(phantom, beam, histories per step, exposures): the 256x256x200 torso at pitch 1.0
    and 40 mm collimation, (big) the 512x512x400 torso at pitch 0.8 and 80 mm, or (c1) the
    DX water cylinder.  count_exposures(beam) -> exposure list (default: the engine's)."""
    from opendxmc_gb300 import phantoms as P

    if count_exposures is None:
        from opendxmc_gb300 import engine as G

        count_exposures = G.beam_exposures

    if c1:
        ph = P.water_cylinder_phantom()
        beam = P.dx_beam_params(particles=1, exposures=10)
    elif big:
        ph = P.torso_phantom(dims=(512, 512, 400), spacing=(0.08, 0.08, 0.1), seed=1)
        beam = P.ct_spiral_params(kvp=120.0, al_mm=6.0, pitch=0.8, collimation_cm=8.0, scan_cm=20.0, particles=1)
    else:
        ph = P.torso_phantom(dims=(256, 256, 200), spacing=(0.15, 0.15, 0.15), seed=1)
        beam = P.ct_spiral_params(kvp=120.0, al_mm=6.0, pitch=1.0, collimation_cm=4.0, scan_cm=20.0, particles=1)
    n_exp = len(count_exposures(beam))
    ppe = int(-(-int(histories) // n_exp))
    beam["particles_per_exposure"] = ppe
    return ph, beam, n_exp * ppe, n_exp


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        loaded = sorted(sm)[len(sm) // 4:] if len(sm) > 4 else sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


def algorithmic_bytes(reads, cell_reads, crossings, deposits) -> float:
    """Bytes the transport must move: 4 B per voxel word read, 4 B per gather-skip
    cell bound read, 4 B per macro-cell crossing (cell scale), 48 B per deposit
    (read-modify-write of the 24-byte tally record)."""
    return 4.0 * reads + 4.0 * cell_reads + 4.0 * crossings + 48.0 * deposits


def cpu_baseline(ph, beam, seconds: float, correction: int = 1) -> dict:
    """The FP64 CPU oracle on this host's cores over a bounded sample of the job:
    consecutive chunks of its histories until `seconds` have passed."""
    from oracle import oracle as O

    O.build()
    threads = os.cpu_count() or 1
    w = O.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials, correction)
    chunk = 2_000_000
    done = 0
    t = time.perf_counter()
    while True:
        st = w.run(beam, seed=1, stream=7, threads=threads, hist_begin=done, hist_end=done + chunk)
        done += st["n_histories"]
        dt = time.perf_counter() - t
        if dt >= seconds or st["n_histories"] < chunk:
            break
    return {"value": done / dt, "unit": "histories/s", "cores": threads, "kind": "port",
            "sample": f"first {done} histories of the same job ({dt:.1f} s, FP64 oracle, {threads} threads)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # the CPU implementation alone: the phantom (numpy) and the oracle's own exposure
    # list; the engine library is neither built nor loaded on this arm
    from oracle import oracle as O

    O.build()
    big = args.workload == "torso512"
    c1 = args.workload == "c1"
    ph, beam, job_hist, _ = workload(args.histories, big, c1, count_exposures=O.beam_exposures)
    threads = os.cpu_count() or 1
    w = O.World(ph.dims, ph.spacing, ph.density, ph.material, ph.materials, args.correction)
    cal = 2_000_000
    t = time.perf_counter()
    w.run(beam, seed=1, threads=threads, hist_end=cal)
    rate = cal / (time.perf_counter() - t)
    per_step = int(min(max(cal, min(rate * 4.0, 2e8)), job_hist))  # ~4 s of CPU work per step
    h = 0

    def sample():
        nonlocal h
        if h + per_step > job_hist:  # wrap around within the job's history range
            h = 0
        st = w.run(beam, seed=1, threads=threads, hist_begin=h, hist_end=h + per_step)
        h += per_step
        return st["n_histories"]

    for _ in range(args.warmup):
        sample()
    t = time.perf_counter()
    done = 0
    for _ in range(args.steps):
        done += sample()
    dt = time.perf_counter() - t
    value = done / dt
    sample = f"{per_step} histories per step of the same job (FP64 oracle port, {threads} threads)"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_C1 if c1 else (WORKLOAD_512 if big else WORKLOAD),
                   "sample_histories_per_step": per_step},
        "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ours(args):
    import numpy as np

    from opendxmc_gb300 import build as B

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    G.set_device(local)
    import torch

    torch.cuda.set_device(local)
    big = args.workload == "torso512"
    c1 = args.workload == "c1"
    ph, beam, hist, n_exp = workload(args.histories, big, c1)
    gw = G.GpuWorld(ph.dims, ph.spacing, ph.materials, args.correction)
    gw.set_data(ph.density, ph.material)
    gw.build()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def run_opts(seed):
        return G.run_options(seed=seed, stream=rank, tracking=TRACKING[args.tracking], macro_cell=args.macro_cell,
                             woodcock_steps=args.woodcock_steps, interact_batch=args.interact_batch,
                             refill_batch=args.refill_batch, gather_skip=args.gather_skip,
                             two_region=args.two_region)

    def step(seed):
        flush.fill_(float(seed))
        torch.cuda.synchronize()
        return gw.run(beam, run_opts(seed))

    for s in range(args.warmup):
        step(1000 + s)
    gw.clear()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    t0 = time.perf_counter()
    stats = [step(1 + s) for s in range(args.steps)]
    barrier()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    if dist is not None:
        tt = torch.tensor([dt], dtype=torch.float64, device=f"cuda:{local}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dt = float(tt.item())
    done = sum(s["n_histories"] for s in stats)
    total_done = done * world
    value = total_done / dt
    kernel_ms = sum(s["kernel_ms"] for s in stats)
    visits = sum(s["n_visits"] for s in stats)
    reads = sum(s["n_voxel_reads"] for s in stats)
    crossings = sum(s["n_crossings"] for s in stats)
    deposits = sum(s["n_photo"] + s["n_compton"] + s["n_cutoff"] for s in stats)
    launches_per_step = -(-hist // LAUNCH_HISTORIES)
    cells = sum(s["n_cell_reads"] for s in stats)
    alg_bytes = algorithmic_bytes(reads, cells, crossings, deposits)
    hbm, peak_kind = peaks()
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "peak_source": peak_kind,
            "traffic": None if c1 else (TRAFFIC_BYTES_PER_HISTORY_512 if big else TRAFFIC_BYTES_PER_HISTORY)
            * hist / launches_per_step,
            "alg_bytes_per_launch": alg_bytes / (args.steps * launches_per_step),
            "kernel_ms_per_launch": kernel_ms / (args.steps * launches_per_step),
            "visits_per_history": visits / done, "voxel_reads_per_history": reads / done,
            "cell_reads_per_history": cells / done,
            "crossings_per_history": crossings / done, "deposits_per_history": deposits / done}

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        N = ph.n_voxels
        dens = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
        mat = torch.empty(N, dtype=torch.uint8, pin_memory=True).numpy()
        dens[:] = ph.density.reshape(-1)
        mat[:] = ph.material.reshape(-1)
        outs = (torch.empty(N, dtype=torch.float64, pin_memory=True).numpy(),
                torch.empty(N, dtype=torch.float64, pin_memory=True).numpy(),
                torch.empty(N, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64))

        def e2e_step(seed):
            gw.set_data(dens, mat)
            gw.build()
            st = gw.run(beam, run_opts(seed))
            gw.dose(out=outs)
            return st

        e2e_step(2000)
        barrier()
        t0 = time.perf_counter()
        hs = sum(e2e_step(3000 + s)["n_histories"] for s in range(args.e2e_steps))
        barrier()
        de = time.perf_counter() - t0
        if dist is not None:
            tt = torch.tensor([de], dtype=torch.float64, device=f"cuda:{local}")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            de = float(tt.item())
        e2e = {"value": hs * world / de, "unit": "histories/s", "h2d_bytes_per_step": N * 9,
               "d2h_bytes_per_step": N * 24, "steps": args.e2e_steps,
               "path": "dxmcg_world_set_data + dxmcg_world_build + dxmcg_transport_run + dxmcg_world_read_dose"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(ph, beam, args.cpu_seconds, args.correction)

    headline = None
    if rank == 0 and world == 1 and args.headline != "none" and not c1:
        headline = time_to_target_headline(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "histories/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD_C1 if c1 else (WORKLOAD_512 if big else WORKLOAD), "grid": list(ph.dims),
                       "voxel_mm": [1.0, 1.0, 2.5] if c1 else ([0.8, 0.8, 1.0] if big else 1.5),
                       "histories_per_step": hist,
                       "exposures": n_exp, "tracking": args.tracking, "correction": args.correction,
                       "macro_cell_voxels": args.macro_cell if args.tracking == "macro" else None, "scoring": "fp64",
                       "l2": "256 MB buffer written before every step" + (
                           "; the 128x128x64 world (5 MB voxels, 34 MB tally) is L2-resident" if c1 else
                           "; tally " + ("3.4 GB" if big else "420 MB") + " > L2"),
                       "parallelism": f"replicas x{world} (independent random streams)"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps, "clocks": clk,
        }
        if headline is not None:
            line["time_to_target"] = headline
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def time_to_target_headline(args) -> dict:
    """Seconds to 2 % RMS dose error (voxels above 10 % of max, judged against two
    independent 1e10-history runs), plain Monte Carlo measured against a short run plus
    the trained denoiser with plain Monte Carlo as the fallback: on the held-out
    512x512x400 spiral-CT torso of the training protocol (120 kVp, pitch 0.8, 80 mm
    collimation) and, with --headline full, on a protocol the network never saw
    (80 kVp, another held-out torso)."""
    import numpy as np
    import torch

    from opendxmc_gb300 import denoise as DN
    from opendxmc_gb300 import engine as G

    wpath = Path(args.weights)
    if not wpath.exists():
        return {"unavailable": f"no trained denoiser parameters at {wpath.name}"}
    net = G.Denoiser((16, 32, 64, 128), seed=0)
    net.set_params(np.load(wpath))
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    dims, spacing = (512, 512, 400), (0.08, 0.08, 0.1)
    out = {"workload": WORKLOAD_512 + "; held-out torso (seed 99), network trained on seeds 11-16",
           "metric": "s to <=2% RMS relative dose error (unbiased against two 1e10-history runs), "
                     "plain MC vs MC + denoiser with plain-MC fallback",
           "weights": wpath.name}
    t0 = time.perf_counter()
    out["c5"] = DN.time_to_target(torch, net, dims, spacing, 99, lambda n: DN.spiral_beam(n), log=log)
    if args.headline == "full":
        out["held_out_protocol"] = DN.time_to_target(
            torch, net, dims, spacing, 98, lambda n: DN.spiral_beam(n, kvp=80.0), log=log)
        out["held_out_protocol"]["protocol"] = "spiral CT 80 kVp 6 mm Al, pitch 0.8, 80 mm (training: 120 kVp)"
    out["wall_s"] = time.perf_counter() - t0
    net.close()
    return out


BATCH_WORKLOAD = ("64 independent DX/CBCT jobs in one persistent launch: seeded six-material ellipsoid phantoms, "
                  "grid 64-320 per axis, 1-3 mm voxels, kVp U(60,140), histories log-U(1e6,1e8) per job")


def run_batch(args):
    """The batched-jobs workload: every job's world resident, one graph-replayed
    launch per step over the shared history queue; beside it the same jobs run one
    dxmcg_transport_run call after another."""
    import numpy as np
    import torch

    from opendxmc_gb300 import build as B
    from opendxmc_gb300 import phantoms as P

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    rank, world, local = dist_env()
    if world > 1:
        raise SystemExit("--workload batch runs on one GPU")
    G.set_device(local)
    torch.cuda.set_device(local)
    specs = P.batched_jobs(n_jobs=64, seed=1)
    t = time.perf_counter()
    worlds = []
    for sp in specs:
        ph = P.ellipsoid_phantom(sp["dims"], sp["spacing"], sp["seed"])
        w = G.GpuWorld(ph.dims, ph.spacing, ph.materials)
        w.set_data(ph.density, ph.material)
        w.build()
        worlds.append(w)
        del ph
    t_setup = time.perf_counter() - t
    trk = TRACKING[args.tracking]
    # autotune on the job with the most histories; its shape drives the batch launch
    n_of = [sp["beam"]["particles_per_exposure"] * sp["beam"].get("n_exposures", 91) for sp in specs]
    big = max(range(len(specs)), key=lambda j: n_of[j])
    t = time.perf_counter()
    tuned, tuned_rate = worlds[big].autotune(specs[big]["beam"], G.run_options(seed=1, tracking=trk,
                                                                                 macro_cell=args.macro_cell))
    t_tune = time.perf_counter() - t

    def opts(j, seed):
        o = G.run_options(seed=seed, stream=j, tracking=trk, macro_cell=args.macro_cell,
                          block_size=tuned.block_size, interact_batch=tuned.interact_batch,
                          refill_batch=tuned.refill_batch, woodcock_steps=tuned.woodcock_steps,
                          gather_skip=args.gather_skip, two_region=args.two_region)
        return o

    batch = G.Batch([(w, sp["beam"], opts(j, 1)) for j, (w, sp) in enumerate(zip(worlds, specs))])
    hist, _ = batch.info()
    total = int(hist.sum())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    def step(s):
        flush.fill_(float(s))
        torch.cuda.synchronize()
        return batch.run()

    for s in range(args.warmup):
        step(s)
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    stats = [step(100 + s) for s in range(args.steps)]
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    done = sum(s["n_histories"] for s in stats)
    kernel_ms = sum(s["kernel_ms"] for s in stats)
    visits = sum(s["n_visits"] for s in stats)
    reads = sum(s["n_voxel_reads"] for s in stats)
    crossings = sum(s["n_crossings"] for s in stats)
    deposits = sum(s["n_photo"] + s["n_compton"] + s["n_cutoff"] for s in stats)
    cells = sum(s["n_cell_reads"] for s in stats)
    alg_bytes = algorithmic_bytes(reads, cells, crossings, deposits)
    hbm, peak_kind = peaks()
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9

    # the same jobs, one transport call each (a separate launch per job, tuned shape)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    seq_done = 0
    for j, (w, sp) in enumerate(zip(worlds, specs)):
        seq_done += w.run(sp["beam"], opts(j, 7))["n_histories"]
    torch.cuda.synchronize()
    seq_dt = time.perf_counter() - t1

    line = {
        "metric": "histories/s", "value": done / dt, "unit": "histories/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "jobs": len(specs), "histories_per_step": total,
                   "voxels": int(sum(int(np.prod(sp["dims"])) for sp in specs)), "tracking": args.tracking,
                   "l2": "256 MB buffer written before every step; tallies 14 GB > L2",
                   "launch": "CUDA graph replayed per step: counter reset + one single-job persistent launch per "
                             "job on 4 streams (a job's blocks take the SMs another job's tail frees)"},
        "autotune": {"block_size": tuned.block_size, "interact_batch": tuned.interact_batch,
                     "refill_batch": tuned.refill_batch, "woodcock_steps": tuned.woodcock_steps,
                     "trial_histories_per_s": tuned_rate, "seconds": t_tune,
                     "job": big},
        "sequential": {"value": seq_done / seq_dt, "unit": "histories/s", "calls": len(specs),
                       "path": "one dxmcg_transport_run per job"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": peak_kind, "traffic": None, "kernel_ms_per_launch": kernel_ms / args.steps},
        # jobs averaging 2^21 histories or more run one single-job launch each in the
        # graph; smaller ones one shared-queue launch (the library's rule)
        "setup_s": t_setup, "gpu_launches": args.steps * (len(specs) if total >= (1 << 21) * len(specs) else 1),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    batch.close()


def run_pipelines(args):
    """The per-voxel passes around the transport on a 512x512x400 volume: CT
    segmentation and the organ dose table on device arrays (kernel time by CUDA
    events, algorithmic bytes vs measured HBM), and the same through the host-array
    entry points (end to end, copies included)."""
    import ctypes as C

    import numpy as np
    import torch

    from opendxmc_gb300 import build as B

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G
    from opendxmc_gb300 import native as N

    G.set_device(0)
    torch.cuda.set_device(0)
    dims = (512, 512, 400)
    n = int(np.prod(dims))
    rng = np.random.default_rng(1)
    hu = np.rint(rng.uniform(-1024.0, 2000.0, n))  # CT numbers are integers
    table = G.ct_segmentation_table(120.0, 2.5, 0.0)
    d_hu = torch.from_numpy(hu).cuda()
    d_mat = torch.empty(n, dtype=torch.uint8, device="cuda")
    d_dens = torch.empty(n, dtype=torch.float64, device="cuda")
    organ = (np.arange(n) // 4096 % 40).astype(np.uint8)
    d_organ = torch.from_numpy(organ).cuda()
    d_dose = torch.rand(n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    sp = np.array([0.08, 0.08, 0.1])
    out = (N.OrganDose * 40)()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    hbm, peak_kind = peaks()

    def timed(fn, reps):
        ms = []
        for r in range(args.warmup + reps):
            flush.fill_(float(r))
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            if r >= args.warmup:
                ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    def seg():
        N.check(N.lib().dxmcg_ct_segment_device(C.byref(table), d_hu.data_ptr(), n, d_mat.data_ptr(),
                                                d_dens.data_ptr(), C.c_void_p(stream.cuda_stream)))

    def organ_table():
        N.check(N.lib().dxmcg_organ_dose_table_device(d_organ.data_ptr(), d_dose.data_ptr(), d_dens.data_ptr(), n,
                                                      N.ptr(sp, C.c_double), 40, out,
                                                      C.c_void_p(stream.cuda_stream)))

    seg_ms = timed(seg, args.steps)
    org_ms = timed(organ_table, args.steps)
    # host arrays through the C ABI (copies in the timed region)
    t = time.perf_counter()
    m_host, d_host = G.ct_segment(table, hu)
    seg_e2e = time.perf_counter() - t
    t = time.perf_counter()
    G.organ_dose_table(organ, hu, d_host, sp, 40)
    org_e2e = time.perf_counter() - t

    def row(bytes_per_voxel, ms, e2e_s):
        gbs = bytes_per_voxel * n / (ms * 1e-3) / 1e9
        return {"voxels_per_s": n / (ms * 1e-3), "kernel_ms": ms, "alg_bytes_per_voxel": bytes_per_voxel,
                "achieved_gbs": gbs, "frac": gbs / hbm, "e2e_voxels_per_s": n / e2e_s, "e2e_s": e2e_s}

    line = {
        "metric": "voxels/s", "value": n / (seg_ms * 1e-3), "unit": "voxels/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "per-voxel passes on a 512x512x400 volume (104,857,600 voxels, integer CT "
                               "numbers uniform in [-1024, 2000])",
                   "l2": "256 MB buffer written before every launch; inputs 0.8-1.8 GB > L2"},
        "peak_gbs": hbm, "peak_source": peak_kind,
        "segmentation": row(17, seg_ms, seg_e2e),
        "organ_dose_table": row(17, org_ms, org_e2e),
    }
    print(json.dumps(line), flush=True)


def run_denoiser(args):
    """Throughput of the denoiser kernels: one training step (batch 8 of 64^3
    patches, channels 16/32/64/128: forward, L1 loss, input and weight gradients,
    Adam) and one forward pass over a 512x512x400 volume; conv FLOPs / CUDA-event
    time against the measured bf16 tensor peak."""
    import torch

    from opendxmc_gb300 import build as B
    from opendxmc_gb300 import denoise as DN

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    G.set_device(0)
    torch.cuda.set_device(0)
    ch = (16, 32, 64, 128)
    net = G.Denoiser(ch, seed=0, conv_path=args.conv_path)
    fwd_per_vox, train_per_vox = DN.conv_flops(ch)
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand((8, 64, 64, 64, 16), device="cuda", generator=gen).to(torch.bfloat16)
    t = torch.rand((8, 64, 64, 64), device="cuda", generator=gen)
    stream = torch.cuda.current_stream()

    def timed(fn, reps):
        ms = []
        for r in range(args.warmup + reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            if r >= args.warmup:
                ms.append(a.elapsed_time(b))
        return statistics.median(ms)

    step_ms = timed(lambda: (net.backward(x, t, stream), net.adam(1e-4, stream)), max(args.steps, 5))
    ix, iy, iz = (int(v) for v in args.inference_dims.split(","))
    vol = torch.rand((1, iz, iy, ix, 16), device="cuda", generator=gen).to(torch.bfloat16)
    out = torch.empty((1, iz, iy, ix), dtype=torch.float32, device="cuda")
    inf_ms = timed(lambda: net.forward(vol, out, stream), max(2, args.steps // 2))
    peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"] if (ROOT / "MEASURED_PEAKS.json").exists() else 1900.0
    step_tf = train_per_vox * 8 * 64 ** 3 / (step_ms * 1e-3) / 1e12
    inf_tf = fwd_per_vox * ix * iy * iz / (inf_ms * 1e-3) / 1e12
    print(json.dumps({
        "metric": "denoiser training step", "value": step_ms, "unit": "ms", "higher_is_better": False, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": "3D conv encoder-decoder 16/32/64/128, batch 8 x 64^3 patches; "
                               f"inference {ix}x{iy}x{iz}"},
        "train_step_ms": step_ms, "train_tflops": step_tf, "train_frac": step_tf / peak,
        "inference_ms": inf_ms, "inference_dims": [ix, iy, iz], "inference_tflops": inf_tf,
        "inference_frac": inf_tf / peak,
        "peak_bf16_tflops": peak, "params": net.n_params,
        "conv_path": {0: "default (tcgen05)", 1: "tcgen05", 2: "mma.sync"}[args.conv_path],
    }), flush=True)


def run_world_denoise(args):
    """Time of the world-path denoiser call (dxmcg_world_denoise: the dose scale, the
    input channels from the tally, the network with its last two convolutions on the
    bricks holding tissue, the dose map left in device memory) on the 512x512x400
    spiral-CT torso after a 3e7-history run.  Untrained weights: the time does not
    depend on them."""
    import torch

    from opendxmc_gb300 import build as B
    from opendxmc_gb300 import denoise as DN
    from opendxmc_gb300 import phantoms as P

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    G.set_device(0)
    torch.cuda.set_device(0)
    dims, spacing = (512, 512, 400), (0.08, 0.08, 0.1)
    ph = P.torso_phantom(dims=dims, spacing=spacing, seed=99)
    world = G.GpuWorld(dims, spacing, [c for _, c, _ in P.SIX_MATERIALS])
    world.set_data(ph.density, ph.material)
    world.build()
    st = world.run(DN.spiral_beam(3e7), G.run_options(seed=5))
    net = G.Denoiser((16, 32, 64, 128), seed=0, conv_path=args.conv_path)
    ms = []
    for r in range(max(args.warmup, 1) + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        net.denoise_world(world, readback=False)
        torch.cuda.synchronize()
        if r >= max(args.warmup, 1):
            ms.append((time.perf_counter() - t0) * 1e3)
    print(json.dumps({
        "metric": "world-path denoiser call", "value": statistics.median(ms), "unit": "ms",
        "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 1),
        "dtype": "bf16", "data": "synthetic",
        "config": {"workload": "512x512x400 spiral-CT torso, 3e7 histories, denoiser 16/32/64/128 (untrained)"},
        "transport_ms": st["total_ms"], "ms_all": ms,
    }), flush=True)


def run_denoise_experiment(args):
    """Seconds to 2 % dose error, plain Monte Carlo vs a short run plus the denoiser,
    on the 512x512x400 spiral-CT torso (trains the network first: a few minutes)."""
    import numpy as np
    import torch

    from opendxmc_gb300 import build as B
    from opendxmc_gb300 import denoise as DN

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    G.set_device(0)
    torch.cuda.set_device(0)
    kw = {}
    if args.small:
        kw = dict(dims=(128, 128, 96), spacing=(0.32, 0.32, 0.4), train_seeds=(11, 12), lows=(1e6, 1e7), high=1e8,
                  steps=60)
    if args.train_steps:
        kw["steps"] = args.train_steps
    if args.lr_final:
        kw["lr_final"] = args.lr_final
    if args.lows:
        kw["lows"] = tuple(float(v) for v in args.lows.split(","))
    if args.init_seeds:
        kw["init_seeds"] = tuple(int(v) for v in args.init_seeds.split(","))
    out, net = DN.experiment(torch, log=lambda m: print(m, file=sys.stderr, flush=True), **kw)
    if args.save_weights:
        np.save(args.save_weights, net.get_params())
    print(json.dumps({"metric": "s to <=2% RMS dose error (plain MC / MC + denoiser)", **out}), flush=True)


def run_c4_training(args):
    """The denoiser trained on Monte-Carlo-generated pairs of 200 seeded 128^3
    six-material phantoms at 2 mm (1e6-history inputs, 1e9-history targets; 64^3
    patches, batch 8, Adam from lr 1e-3, L1 loss), then scored on held-out phantoms."""
    import numpy as np
    import torch

    from opendxmc_gb300 import build as B
    from opendxmc_gb300 import denoise as DN

    if not B.LIB.exists():
        B.build(verbose_ptxas=False)
    from opendxmc_gb300 import engine as G

    G.set_device(0)
    torch.cuda.set_device(0)
    kw = {"n_phantoms": args.phantoms}
    if args.train_steps:
        kw["steps"] = args.train_steps
    out, net = DN.c4_experiment(torch, log=lambda m: print(m, file=sys.stderr, flush=True), **kw)
    if args.save_weights:
        np.save(args.save_weights, net.get_params())
    print(json.dumps({"metric": "denoiser trained on 200 phantoms of 128^3 (1e6 / 1e9-history pairs): held-out "
                                "RMS relative dose error, input vs denoised", **out}), flush=True)


def main():
    args = parse()
    if args.workload == "c1" and args.histories == 1e9:
        args.histories = 1e7  # the configuration's history count
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "pipelines":
        run_pipelines(args)
    elif args.workload == "denoiser":
        run_denoiser(args)
    elif args.workload == "world-denoise":
        run_world_denoise(args)
    elif args.workload == "denoise-experiment":
        run_denoise_experiment(args)
    elif args.workload == "c4-training":
        run_c4_training(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
