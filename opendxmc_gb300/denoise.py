"""Training data, training loop and evaluation of the dose denoiser.

The data come from the GPU transport itself: for each seeded phantom a short run
(the network's input) and a long run (its target) of the same beam with
independent random streams.  Inputs are normalised by the short run's mean dose
over voxels denser than 0.2 g/cm3; targets are the long run's dose over the same
scale.  Everything stays in device memory (CUDA tensors; torch is the container),
and every operation on it is a library kernel: transport, input preparation, patch
gathering, forward, backward, Adam.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass

import numpy as np

from . import engine as G
from . import native as N


def conv_flops(channels, in_channels=16):
    """Multiply-add FLOPs per output voxel of level 0 for one forward pass, and the
    same for one training step (forward + input gradients + weight gradients)."""
    L = len(channels)
    fwd = 0.0
    dgrad = 0.0
    prev = in_channels
    for l, c in enumerate(channels):
        scale = 1.0 / 8 ** l
        for k, (ci, co) in enumerate([(prev, c), (c, c)]):
            f = 2 * 27 * ci * co * scale
            fwd += f
            if not (l == 0 and k == 0):
                dgrad += f
        prev = c
    for l in range(L - 2, -1, -1):
        scale = 1.0 / 8 ** l
        for ci, co in [(channels[l + 1] + channels[l], channels[l]), (channels[l], channels[l])]:
            f = 2 * 27 * ci * co * scale
            fwd += f
            dgrad += f
    return fwd, 2 * fwd + dgrad  # training: forward + weight gradients (= forward) + input gradients


@dataclass
class Pair:
    """One training volume on the device."""
    input: object   # bf16 [D, H, W, 16]
    target: object  # float32 [D, H, W]
    scale: float
    dims: tuple     # (D, H, W)


def dose_pair(world: "G.GpuWorld", beam: dict, low: int, high: int, seed: int, stream_base: int = 0):
    """(low-history dose, high-history dose) of one beam on one world, mGy per voxel
    (host arrays); the two runs use independent random streams."""
    def run(n, stream):
        b = dict(beam)
        world.clear()
        ppe = max(1, int(round(n / _exposures(b))))
        b["particles_per_exposure"] = ppe
        world.run(b, G.run_options(seed=seed, stream=stream))
        return world.dose()[0]

    d_low = run(low, stream_base)
    d_high = run(high, stream_base + 1)
    return d_low, d_high


def _exposures(beam: dict) -> int:
    return len(G.beam_exposures(dict(beam, particles_per_exposure=1)))


def make_pair(torch, world: "G.GpuWorld", dims_zyx, d_low, d_high, rho, mat, ratio: float = 1.0) -> Pair:
    """Input from the short run, target = the long run's dose x `ratio` (= short /
    long history count: dose is not normalised per history, so this puts the
    target in the short run's units), both over the short run's scale."""
    sel = rho > 0.2
    scale = float(d_low[sel].mean()) if sel.any() and d_low[sel].mean() > 0 else float(d_low.mean() or 1.0)
    dev = "cuda"
    x = G.prepare_input(torch.tensor(d_low.reshape(dims_zyx), dtype=torch.float32, device=dev),
                        torch.tensor(rho.reshape(dims_zyx), dtype=torch.float32, device=dev),
                        torch.tensor(mat.reshape(dims_zyx), dtype=torch.uint8, device=dev), scale)
    t = torch.tensor((d_high * (ratio / scale)).reshape(dims_zyx), dtype=torch.float32, device=dev)
    return Pair(x, t, scale, tuple(dims_zyx))


class PatchSampler:
    """Random patch origins over a list of Pairs; gathers batches on the device.
    With `centers` (per pair, an array of (z, y, x) voxels) a fraction `focus` of the
    patches is centred on one of them (e.g. the body), the rest anywhere."""

    def __init__(self, torch, pairs: list[Pair], patch: int, batch: int, seed: int = 0, centers=None,
                 focus: float = 0.9):
        self.torch = torch
        self.pairs = pairs
        self.P = patch
        self.B = batch
        self.rng = np.random.default_rng(seed)
        self.centers = centers
        self.focus = focus
        dev = "cuda"
        self.ptr_in = torch.tensor([p.input.data_ptr() for p in pairs], dtype=torch.int64, device=dev)
        self.ptr_t = torch.tensor([p.target.data_ptr() for p in pairs], dtype=torch.int64, device=dev)
        self.dims = torch.tensor(np.array([p.dims for p in pairs]).ravel(), dtype=torch.int32, device=dev)
        self.xb = torch.empty((batch, patch, patch, patch, 16), dtype=torch.bfloat16, device=dev)
        self.tb = torch.empty((batch, patch, patch, patch), dtype=torch.float32, device=dev)

    def sample(self):
        org = np.zeros((self.B, 4), dtype=np.int32)
        for k in range(self.B):
            v = int(self.rng.integers(len(self.pairs)))
            D, H, W = self.pairs[v].dims
            if self.centers is not None and len(self.centers[v]) and self.rng.random() < self.focus:
                c = self.centers[v][self.rng.integers(len(self.centers[v]))]
                h = self.P // 2
                org[k] = (v, min(max(c[0] - h, 0), D - self.P), min(max(c[1] - h, 0), H - self.P),
                          min(max(c[2] - h, 0), W - self.P))
            else:
                org[k] = (v, self.rng.integers(0, D - self.P + 1), self.rng.integers(0, H - self.P + 1),
                          self.rng.integers(0, W - self.P + 1))
        o = self.torch.tensor(org.ravel(), dtype=self.torch.int32, device="cuda")
        N.check(N.lib().dxmcg_denoiser_gather_patches(C.c_void_p(self.ptr_in.data_ptr()),
                                                      C.c_void_p(self.ptr_t.data_ptr()),
                                                      C.c_void_p(self.dims.data_ptr()), len(self.pairs),
                                                      C.c_void_p(o.data_ptr()), self.B, self.P,
                                                      C.c_void_p(self.xb.data_ptr()), C.c_void_p(self.tb.data_ptr()),
                                                      None))
        return self.xb, self.tb


def train(net: "G.Denoiser", sampler: PatchSampler, steps: int, lr: float = 1e-3, log_every: int = 0,
          lr_final: float | None = None, log=print):
    """Adam on random patches; returns the loss of every `every`-th step (reading the
    loss back waits for the GPU, so it is not read on the others).  With lr_final the
    rate decays geometrically from lr to lr_final."""
    losses = []
    every = max(1, log_every // 20) if log_every else 16  # read the loss back on these steps only
    for s in range(steps):
        rate = lr if lr_final is None else lr * (lr_final / lr) ** (s / max(1, steps - 1))
        x, t = sampler.sample()
        loss = net.train_step(x, t, rate, want_loss=(s % every == every - 1) or s == steps - 1)
        if loss is not None:
            losses.append(loss)
        if log_every and (s + 1) % log_every == 0:
            log(f"step {s + 1}: loss {np.mean(losses[-20:]):.4f}")
    return losses


def relative_errors(estimate, reference, reference2=None, threshold=0.1, mask=None):
    """Errors over voxels whose reference dose exceeds `threshold` x its maximum:
    mean |e - r| / r against the reference, and, with a second independent
    reference, the RMS relative error with the references' own noise removed:
    E[(e - r1)(e - r2)] = E[(e - truth)^2] when r1 and r2 are independent of e and
    of each other."""
    ref = reference if reference2 is None else 0.5 * (reference + reference2)
    cand = ref if mask is None else np.where(mask, ref, 0.0)
    sel = cand > threshold * cand.max()
    e = estimate[sel]
    out = {"voxels": int(sel.sum()), "mean_rel": float(np.mean(np.abs(e - ref[sel]) / ref[sel]))}
    if reference2 is not None:
        r1 = reference[sel]
        r2 = reference2[sel]
        cross = (e - r1) * (e - r2) / (ref[sel] ** 2)
        out["rms_rel_unbiased"] = float(np.sqrt(max(np.mean(cross), 0.0)))
        # the references' own RMS relative noise: E[(r1 - r2)^2] / 2
        out["reference_rms_rel"] = float(np.sqrt(np.mean((r1 - r2) ** 2 / (ref[sel] ** 2)) / 2))
    return out


class Scorer:
    """Errors of a dose map against two independent reference runs r1 and r2 (same
    units), over the voxels that are not air and whose averaged reference dose exceeds
    `threshold` x its maximum:

      rms_rel         RMS relative error with the references' own noise removed:
                      E[(e - r1)(e - r2)] = E[(e - truth)^2] for r1, r2 independent of e
                      and of each other;
      mean_rel        mean |e - rbar| / rbar against the references' average rbar;
      mean_rel_floor  that statistic for an exact map, mean |r1 - r2| / (2 rbar): rbar's
                      own noise, below which mean_rel cannot go whatever the estimate."""

    def __init__(self, r1, r2, nonair, threshold=0.1):
        rbar = 0.5 * (r1 + r2)
        cand = np.where(nonair, rbar, 0.0)
        self.sel = np.flatnonzero(cand > threshold * cand.max())
        self.r1 = r1[self.sel]
        self.r2 = r2[self.sel]
        self.rbar = rbar[self.sel]
        self.floor = float(np.mean(np.abs(self.r1 - self.r2) / (2.0 * self.rbar)))
        self.reference_rms = float(np.sqrt(np.mean((self.r1 - self.r2) ** 2 / self.rbar ** 2) / 2))

    def __call__(self, estimate) -> dict:
        e = estimate[self.sel]
        cross = (e - self.r1) * (e - self.r2) / self.rbar ** 2
        return {"rms_rel": float(np.sqrt(max(np.mean(cross), 0.0))),
                "mean_rel": float(np.mean(np.abs(e - self.rbar) / self.rbar)),
                "mean_rel_floor": self.floor, "voxels": int(self.sel.size)}


def plain_to_target(world, beam_of, high, scorer, target, air, seed, chunk, start, limit, stream0=100, log=print):
    """Plain Monte Carlo, measured: runs of `chunk` histories on independent streams
    add up in the world's tally until the error of the accumulated map (scaled to the
    `high`-history references) crosses `target`; the map is scored after every run
    once `start` histories are in (reading it back is not timed).  Returns the checks,
    the first passing one, and the crossing N* = N (rms / target)^2 of that check
    (rms^2 falls as 1/N for plain Monte Carlo), with its time at the measured rate."""
    world.clear()
    n, mc_s, k = 0, 0.0, 0
    checks = []
    while n < limit:
        st = world.run(beam_of(chunk), G.run_options(seed=seed, stream=stream0 + k))
        k += 1
        n += st["n_histories"]
        mc_s += st["total_ms"] * 1e-3
        if n < start:
            continue
        d = world.dose()[0]
        d[air] = 0.0
        e = scorer(d * (high / n))
        checks.append({"histories": n, "mc_s": mc_s, **e})
        log(f"plain MC {n:.3g} histories, {mc_s:.2f} s: RMS {e['rms_rel']:.4f}, mean {e['mean_rel']:.4f}")
        if e["rms_rel"] <= target:
            break
    last = checks[-1] if checks else None
    passed = last is not None and last["rms_rel"] <= target
    out = {"checks": checks, "passed": passed, "histories_per_s": n / mc_s if mc_s > 0 else None}
    if passed:
        n_star = last["histories"] * (last["rms_rel"] / target) ** 2
        out.update({"histories": last["histories"], "s": last["mc_s"], "rms_rel": last["rms_rel"],
                    "mean_rel": last["mean_rel"], "crossing_histories": n_star,
                    "crossing_s": n_star / out["histories_per_s"]})
    return out


def denoised_to_target(torch, world, net, beam_of, high, scorer, target, lows, air, seed, stream0=20,
                       log=print):
    """A short run plus the denoiser, judged by the references: inputs of each history
    count in `lows` in turn, each attempt's time (transport + inference, the denoised
    map left in device memory) added to the total, until one denoised map meets
    `target`.  When none does, the caller falls back on plain Monte Carlo."""
    total = 0.0
    attempts = []
    for k, low in enumerate(lows):
        world.clear()
        st = world.run(beam_of(low), G.run_options(seed=seed, stream=stream0 + k))
        t_mc = st["total_ms"] * 1e-3
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        net.denoise_world(world, readback=False)
        torch.cuda.synchronize()
        t_inf = time.perf_counter() - t1
        d_dn, _ = net.denoise_world(world)  # the same map again, read back for scoring
        d_dn[air] = 0.0
        e = scorer(d_dn * (high / low))
        d_in = world.dose()[0]
        d_in[air] = 0.0
        e_in = scorer(d_in * (high / low))
        total += t_mc + t_inf
        ok = e["rms_rel"] <= target
        attempts.append({"histories": low, "mc_s": t_mc, "inference_s": t_inf, "rms_rel": e["rms_rel"],
                         "mean_rel": e["mean_rel"], "input_rms_rel": e_in["rms_rel"], "accepted": ok})
        log(f"{low:.3g} histories + denoiser: RMS {e['rms_rel']:.4f} (input {e_in['rms_rel']:.4f}), "
            f"{'accepted' if ok else 'rejected'}")
        if ok:
            return {"accepted": True, "histories": low, "s": total, "rms_rel": e["rms_rel"],
                    "mean_rel": e["mean_rel"], "attempts": attempts}
    return {"accepted": False, "s": total, "attempts": attempts}


def time_to_target(torch, net, dims, spacing, phantom_seed, beam_of, high=1e10, target=0.02,
                   lows=(3e7, 1e8, 3e8, 1e9), plain_chunk=1e10, log=print):
    """Seconds to `target` RMS relative dose error on one torso: plain Monte Carlo
    (measured, plain_to_target) against a short run plus the denoiser with plain Monte
    Carlo as the fallback (denoised_to_target), both judged against two independent
    `high`-history runs over non-air voxels above 10 % of the maximum dose."""
    from . import phantoms as P

    t0 = time.perf_counter()
    ph = P.torso_phantom(dims=dims, spacing=spacing, seed=phantom_seed)
    world = G.GpuWorld(dims, spacing, [c for _, c, _ in P.SIX_MATERIALS])
    world.set_data(ph.density, ph.material)
    world.build()
    del ph
    _, mat = world.packed_density()
    air = mat == 0
    refs = []
    for stream in (2, 3):
        world.clear()
        world.run(beam_of(high), G.run_options(seed=phantom_seed, stream=stream))
        d = world.dose()[0]
        d[air] = 0.0
        refs.append(d)
    scorer = Scorer(refs[0], refs[1], ~air)
    del refs
    t_setup = time.perf_counter() - t0
    log(f"references: 2 x {high:.3g} histories, RMS noise {scorer.reference_rms:.4f}, "
        f"mean-error floor {scorer.floor:.4f}, {scorer.sel.size} voxels scored")
    world.clear()
    world.run(beam_of(lows[0]), G.run_options(seed=phantom_seed, stream=9))
    net.denoise_world(world, readback=False)  # sizes the network's buffers for this grid
    dn = denoised_to_target(torch, world, net, beam_of, high, scorer, target, lows, air, phantom_seed, log=log)
    n_pred = high * (scorer.reference_rms / target) ** 2
    plain = plain_to_target(world, beam_of, high, scorer, target, air, phantom_seed, chunk=plain_chunk,
                            start=0.6 * n_pred, limit=3.0 * n_pred, log=log)
    if not dn["accepted"] and plain["passed"]:
        dn["fallback_plain_s"] = plain["s"]
        dn["s"] += plain["s"]
    world.close()
    out = {"reference_histories": high, "reference_rms_rel": scorer.reference_rms,
           "mean_rel_floor": scorer.floor, "voxels_scored": int(scorer.sel.size), "target_rms_rel": target,
           "plain": plain, "denoised": dn, "setup_s": t_setup}
    if plain["passed"]:
        out["speedup_vs_plain_crossing"] = plain["crossing_s"] / dn["s"]
    return out


# ---------------------------------------------------------------- the spiral-CT experiment
def spiral_beam(histories: float, pitch=0.8, collimation_cm=8.0, scan_cm=20.0, kvp=120.0, al_mm=6.0) -> dict:
    from . import phantoms as P

    b = P.ct_spiral_params(kvp=kvp, al_mm=al_mm, pitch=pitch, collimation_cm=collimation_cm, scan_cm=scan_cm,
                           particles=1)
    n_exp = _exposures(b)
    b["particles_per_exposure"] = max(1, int(np.ceil(histories / n_exp)))
    return b


def run_dose(world, beam, seed, stream, air):
    """One transport run from a cleared tally: (dose with air zeroed, stats)."""
    world.clear()
    st = world.run(beam, G.run_options(seed=seed, stream=stream))
    d = world.dose()[0]
    d[air] = 0.0
    return d, st


def experiment(torch, dims=(512, 512, 400), spacing=(0.08, 0.08, 0.1), train_seeds=(11, 12, 13, 14, 15, 16),
               eval_seed=99, lows=(3e7, 1e8, 3e8, 1e9), high=1e10, steps=16000, batch=8, patch=64, lr=1e-3,
               lr_final=5e-5, channels=(16, 32, 64, 128), target_error=0.02, init_seeds=(0,), val_seed=97,
               log=print):
    """Train the denoiser on torso phantoms (inputs: runs of each history count in
    `lows`; target: a `high`-history run), then, on a held-out torso, compare the
    time to `target_error` of plain Monte Carlo with that of a short run plus
    denoising, for each input history count.  Error: RMS relative error over
    non-air voxels above 10 % of the maximum dose, made unbiased by two independent
    `high`-history references; plain Monte Carlo's error at N histories is one
    reference's own noise scaled by sqrt(high / N).

    With several `init_seeds` one network is trained from each initialisation and the
    one with the lowest error at the smallest input (then the next) on a validation
    torso (`val_seed`, neither a training nor the evaluation torso) is kept: the
    evaluation torso plays no part in the choice."""
    from . import phantoms as P

    nx, ny, nz = dims
    beam_high = spiral_beam(high)
    world = G.GpuWorld(dims, spacing, [c for _, c, _ in P.SIX_MATERIALS])
    pairs, centers = [], []
    t0 = time.perf_counter()
    mc_s = 0.0
    for s in train_seeds:
        ph = P.torso_phantom(dims=dims, spacing=spacing, seed=s)
        world.set_data(ph.density, ph.material)
        world.build()
        rho, mat = world.packed_density()
        air = mat == 0
        d_high, st = run_dose(world, beam_high, s, 1, air)
        mc_s += st["total_ms"] * 1e-3
        body = np.flatnonzero(rho > 0.2)
        pick = np.random.default_rng(s).choice(body, size=min(200_000, body.size), replace=False)
        c = np.stack(np.unravel_index(pick, (nz, ny, nx)), axis=1)
        for k, low in enumerate(lows):
            d_low, st = run_dose(world, spiral_beam(low), s, 10 + k, air)
            mc_s += st["total_ms"] * 1e-3
            pairs.append(make_pair(torch, world, (nz, ny, nx), d_low, d_high, rho, mat, low / high))
            centers.append(c)
        log(f"phantom {s}: {len(lows)} inputs, target {high:.3g} histories, scale {pairs[-1].scale:.4g}")
    t_data = time.perf_counter() - t0

    sampler = PatchSampler(torch, pairs, patch, batch, seed=1, centers=centers)
    candidates = []
    t_train = 0.0
    for init in init_seeds:
        cand = G.Denoiser(channels, seed=init)
        sampler.rng = np.random.default_rng(1)  # every candidate sees the same patches
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cand_losses = train(cand, sampler, steps, lr=lr, lr_final=lr_final, log_every=max(1, steps // 10), log=log)
        torch.cuda.synchronize()
        t_train += time.perf_counter() - t0
        candidates.append((cand, cand_losses))
    del sampler, pairs

    validation = []
    if len(candidates) > 1:
        ph = P.torso_phantom(dims=dims, spacing=spacing, seed=val_seed)
        world.set_data(ph.density, ph.material)
        world.build()
        _, mat = world.packed_density()
        air = mat == 0
        v1, _ = run_dose(world, beam_high, val_seed, 2, air)
        v2, _ = run_dose(world, beam_high, val_seed, 3, air)
        scorer = Scorer(v1, v2, ~air)
        for k, low in enumerate(lows):
            run_dose(world, spiral_beam(low), val_seed, 20 + k, air)
            errs = []
            for cand, _ in candidates:
                d_dn, _ = cand.denoise_world(world)
                d_dn[air] = 0.0
                errs.append(scorer(d_dn * (high / low))["rms_rel"])
            validation.append(errs)
        for i, init in enumerate(init_seeds):
            log(f"candidate {init}: validation RMS " + ", ".join(f"{v[i]:.4f}" for v in validation))
    order = sorted(range(len(candidates)), key=lambda i: tuple(v[i] for v in validation))
    chosen = order[0]
    net, losses = candidates[chosen]
    for i, (cand, _) in enumerate(candidates):
        if i != chosen:
            cand.close()

    # held-out torso
    ph = P.torso_phantom(dims=dims, spacing=spacing, seed=eval_seed)
    world.set_data(ph.density, ph.material)
    world.build()
    rho, mat = world.packed_density()
    air = mat == 0
    nonair = ~air
    r1, s_r1 = run_dose(world, beam_high, eval_seed, 2, air)
    r2, _ = run_dose(world, beam_high, eval_seed, 3, air)
    rate = s_r1["n_histories"] / (s_r1["total_ms"] * 1e-3)
    levels = []
    sigma_ref = None
    for k, low in enumerate(lows):
        d_low, s_low = run_dose(world, spiral_beam(low), eval_seed, 20 + k, air)
        net.denoise_world(world, readback=False)  # first call sizes the network's buffers
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        net.denoise_world(world, readback=False)  # the denoised map, on the device like the MC tally
        t_inf = time.perf_counter() - t1
        t1 = time.perf_counter()
        d_dn, scale = net.denoise_world(world)  # again, read back for scoring
        t_inf_host = time.perf_counter() - t1
        d_dn[air] = 0.0
        d_dn *= high / low  # in the references' units
        e_dn = relative_errors(d_dn, r1, r2, mask=nonair)
        e_low = relative_errors(d_low * (high / low), r1, r2, mask=nonair)
        sigma_ref = e_dn["reference_rms_rel"]
        t_low = s_low["total_ms"] * 1e-3
        levels.append({"histories": low, "mc_s": t_low, "inference_s": t_inf,
                       "inference_with_readback_s": t_inf_host, "total_s": t_low + t_inf,
                       "low_rms_rel": e_low["rms_rel_unbiased"], "denoised_rms_rel": e_dn["rms_rel_unbiased"],
                       "denoised_mean_rel": e_dn["mean_rel"], "voxels_scored": e_dn["voxels"],
                       "meets_target": bool(e_dn["rms_rel_unbiased"] <= target_error)})
        log(f"eval {low:.3g}: denoised RMS {e_dn['rms_rel_unbiased']:.4f}, input RMS {e_low['rms_rel_unbiased']:.4f}")
    n_plain = high * (sigma_ref / target_error) ** 2
    t_plain = n_plain / rate
    ok = [lv for lv in levels if lv["meets_target"]]
    best = min(ok, key=lambda lv: lv["total_s"]) if ok else None
    out = {
        "dims": list(dims), "spacing_cm": list(spacing), "train_phantoms": len(train_seeds), "inputs": list(lows),
        "high": high, "train_steps": steps, "batch": batch, "patch": patch,
        "final_loss": float(np.mean(losses[-10:])), "data_s": t_data, "data_mc_s": mc_s, "train_s": t_train,
        "init_seeds": list(init_seeds), "chosen_init_seed": init_seeds[chosen], "validation_seed": val_seed,
        "validation_rms_rel": validation,
        "histories_per_s": rate, "reference_rms_rel": sigma_ref, "target_error": target_error,
        "plain_histories_to_target": n_plain, "plain_s_to_target": t_plain, "levels": levels,
        "denoised_s_to_target": best["total_s"] if best else None,
        "denoised_histories": best["histories"] if best else None,
        "speedup": t_plain / best["total_s"] if best else None,
    }
    return out, net


# ---------------------------------------------------------------- training on many small phantoms
def c4_experiment(torch, n_phantoms=200, dims=(128, 128, 128), spacing=(0.2, 0.2, 0.2), low=1e6, high=1e9,
                  eval_phantoms=10, steps=16000, batch=8, patch=64, lr=1e-3, lr_final=5e-5,
                  channels=(16, 32, 64, 128), seed0=5000, log=print):
    """The denoiser trained on data the Monte Carlo generates from many small
    phantoms: `n_phantoms` seeded six-material ellipsoid phantoms of `dims` voxels,
    each run for `low` histories (input) and `high` histories (target) with independent
    streams, spiral CT 120 kVp / 6 mm Al with the body bowtie, pitch 1.0, 40 mm
    collimation over the phantom's length.  Then, on `eval_phantoms` held-out phantoms
    of the same generator, the RMS relative error of the input and of its denoised map
    against two independent `high`-history runs (non-air voxels above 10 % of max)."""
    from . import phantoms as P

    nx, ny, nz = dims
    length = nz * spacing[2]

    def beam_of(n):
        return spiral_beam(n, pitch=1.0, collimation_cm=4.0, scan_cm=length)

    mats = [c for _, c, _ in P.SIX_MATERIALS]
    world = G.GpuWorld(dims, spacing, mats)
    pairs, centers = [], []
    t0 = time.perf_counter()
    mc_s, hist = 0.0, 0
    for i in range(n_phantoms):
        ph = P.ellipsoid_phantom(dims, spacing, seed=seed0 + i)
        world.set_data(ph.density, ph.material)
        world.build()
        rho, mat = world.packed_density()
        air = mat == 0
        d_high, st = run_dose(world, beam_of(high), seed0 + i, 1, air)
        mc_s += st["total_ms"] * 1e-3
        hist += st["n_histories"]
        d_low, st = run_dose(world, beam_of(low), seed0 + i, 10, air)
        mc_s += st["total_ms"] * 1e-3
        hist += st["n_histories"]
        pairs.append(make_pair(torch, world, (nz, ny, nx), d_low, d_high, rho, mat, low / high))
        body = np.flatnonzero(rho > 0.2)
        pick = np.random.default_rng(i).choice(body, size=min(20_000, body.size), replace=False)
        centers.append(np.stack(np.unravel_index(pick, (nz, ny, nx)), axis=1))
        if (i + 1) % 20 == 0:
            log(f"phantom {i + 1}/{n_phantoms}: {hist:.3g} histories in {mc_s:.1f} s of transport")
    t_data = time.perf_counter() - t0

    net = G.Denoiser(channels, seed=0)
    sampler = PatchSampler(torch, pairs, patch, batch, seed=1, centers=centers)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = train(net, sampler, steps, lr=lr, lr_final=lr_final, log_every=max(1, steps // 10), log=log)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del sampler, pairs

    evals = []
    for i in range(eval_phantoms):
        s = seed0 + n_phantoms + 1000 + i
        ph = P.ellipsoid_phantom(dims, spacing, seed=s)
        world.set_data(ph.density, ph.material)
        world.build()
        _, mat = world.packed_density()
        air = mat == 0
        r1, _ = run_dose(world, beam_of(high), s, 2, air)
        r2, _ = run_dose(world, beam_of(high), s, 3, air)
        scorer = Scorer(r1, r2, ~air)
        d_low, st = run_dose(world, beam_of(low), s, 20, air)
        d_dn, _ = net.denoise_world(world)
        d_dn[air] = 0.0
        e_in = scorer(d_low * (high / low))
        e_dn = scorer(d_dn * (high / low))
        evals.append({"seed": s, "input_rms_rel": e_in["rms_rel"], "denoised_rms_rel": e_dn["rms_rel"],
                      "input_mean_rel": e_in["mean_rel"], "denoised_mean_rel": e_dn["mean_rel"],
                      "mean_rel_floor": e_dn["mean_rel_floor"], "reference_rms_rel": scorer.reference_rms})
        log(f"held-out phantom {s}: input RMS {e_in['rms_rel']:.3f}, denoised RMS {e_dn['rms_rel']:.4f}")
    world.close()
    return {
        "phantoms": n_phantoms, "dims": list(dims), "spacing_cm": list(spacing), "low": low, "high": high,
        "train_steps": steps, "batch": batch, "patch": patch, "lr": lr, "lr_final": lr_final,
        "final_loss": float(np.mean(losses[-10:])), "first_loss": float(np.mean(losses[:5])),
        "data_s": t_data, "data_mc_s": mc_s, "data_histories": hist, "train_s": t_train,
        "held_out": evals,
        "mean_input_rms_rel": float(np.mean([e["input_rms_rel"] for e in evals])),
        "mean_denoised_rms_rel": float(np.mean([e["denoised_rms_rel"] for e in evals])),
    }, net
