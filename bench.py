"""Benchmark of the AMOEBA induce() hot path on one GB300 (replicas for N>1).

A step is one induce() call -- permanent field (PME + real space), PCG to a
1e-6 Debye RMS residual with the sparse preconditioner and the ASPC predictor
-- on one frame of a seeded 1 fs trajectory of the 12,288-atom AMOEBA water
box (49.31 A, PME 64^3, order 5, a = 0.5446, 7 A cutoff).  Frames are
synthetic: molecules librate and rattle about seeded lattice sites, so the
induce legs time the same coordinates on every run.  The MD leg (ns/day)
integrates the same box with the whole water force field.

value: induce() calls per second over all ranks, inputs resident in HBM
       (the librating trajectory; induce_md_frames repeats the solve on
       frames of the MD leg's trajectory of the relaxed box).
e2e:   the same through t9gb_induce_host: host coordinates in, host dipoles
       out, both copies inside the timed region.
*_learned_extrapolation: the librating, MD-frame, 98,304-atom and MD legs
       again with the ASPC ring's coefficients fitted online after every solve
       (t9gb_learn_extrapolation, LX_ORDER frames) instead of ASPC's own.
learned_guess: the per-atom network's starts on MD frames against the plain
       ones (alpha E and ASPC).
The working set (~10 MB) is smaller than L2, so L2 is flushed (a 512 MB
write) between timed steps, outside the per-step CUDA-event brackets.

--impl reference times the CPU implementation of the same step: the FP64 C
restatement of the reference's host path (oracle/), all host threads, on the
same frames and from the same ASPC start (16 untimed history solves first).
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "AMOEBA water ns/day & induce ms/step, learned vs plain PCG at 1e-6 D, 1 GB300"
WORKLOAD = "water12288"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=WORKLOAD)
    ap.add_argument("--predictor", default="aspc", choices=["aspc", "none"])
    ap.add_argument("--history", type=int, default=20, help="trajectory frames run before warm-up (predictor ring)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--learn-train", type=int, default=500, help="online training steps before the learned legs")
    ap.add_argument("--learn-steps", type=int, default=1500,
                    help="timed steps per learned leg on the 12,288-atom MD frames (the network in use on steps "
                    "500-2000 of the learned-guess configuration)")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-forces", action="store_true")
    ap.add_argument("--no-md", action="store_true", help="skip the MD leg (ns/day)")
    ap.add_argument("--md-steps", type=int, default=1000, help="timed MD steps (after 2 ps of relaxation)")
    ap.add_argument("--md-extra", default="nacl23142,water98304",
                    help="further configurations timed as MD (comma separated; empty: none)")
    ap.add_argument("--no-large", action="store_true", help="skip the 98,304-atom leg")
    ap.add_argument("--large-config", default="water98304")
    ap.add_argument("--fft", choices=["auto", "own", "cufft"], default="auto",
                    help="PME transform: the library's default (its fused transform on cubic 32/64 grids, cuFFT "
                    "otherwise), the fused transform, or cuFFT")
    ap.add_argument("--lanes", type=int, default=0,
                    help="lanes per atom in the real-space field kernels (0: the library's choice by box size)")
    ap.add_argument("--no-flush", action="store_true",
                    help="skip the 512 MB L2 flush buffer (for ncu captures only; numbers are not bench values)")
    ap.add_argument("--stepwise", action="store_true",
                    help="learned legs without CUDA graphs, so that ncu sees each launch (numbers are not bench values)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
            )
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
            "power_w_max": max(power) if power else None,
        }


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# Algorithmic (compulsory) bytes per launch of each kernel: every input read
# once, every output written once.  "entries" = neighbour-list entries.
def algorithmic_bytes(kernel, n, entries, nfft):
    ng = nfft ** 3
    if kernel == "ufield_real":
        # pos 16 + dipoles 24 + damping 8 + recip field 24 in, field 24 out, list 4/entry
        return n * (16 + 24 + 8 + 24 + 24) + 4 * entries
    if kernel == "dfield_real":
        # pos 16 + multipoles 40 + damping 8 + recip field 24 in, field 24 out
        return n * (16 + 40 + 8 + 24 + 24) + 4 * entries
    if kernel == "precond_sparse":
        return n * (16 + 24 + 8 + 4 + 24) + 4 * entries
    if kernel == "spread_uind":
        # pos + dipoles in, fixed-point grid (one 8-byte word per point: d and p packed) written once
        return n * (16 + 24) + 8 * ng
    if kernel == "spread_mpole":
        return n * (16 + 40) + 8 * ng
    if kernel == "fft_conv":
        # compulsory traffic of one transform + convolution: the packed fixed-point grid read (8 B/pt) and
        # cleared (8), the influence table read (4), the complex grid written for the gather (8); the
        # intermediate passes of the transform are not compulsory (FFT_PASS_BYTES)
        return ng * (8 + 8 + 4 + 8)
    if kernel in ("gather_uind", "gather_mpole"):
        return 8 * ng + n * (16 + 24 + 24)
    if kernel == "pcg_vector":
        # per iteration: direction (3 vectors), Ap (3 + 1/alpha), update (6): 4 vectors of 6 floats per launch
        return n * 6 * 4 * 4
    if kernel == "nblist":
        return n * 16 + 4 * entries
    return n * 16


# Bytes a three-pass transform also moves between its passes (complex grid
# written and read by the plane, z-line and plane passes): reported beside the
# compulsory figure, not counted in it.
FFT_PASS_BYTES = 8 + 8 + 8 + 8


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of a
# kernel group, from one `ncu --set full --clock-control none` capture on
# GB300 of `bench.py --steps 3 --warmup 3 --no-learned --no-large
# --no-cpu-baseline --no-flush --no-md` (water12288, fused 64^3 transform):
# the dipole transform + convolution is k_fft_plane<64,1,0> 2,112,000 +
# k_fft_zline<64,2> 3,158,528 + k_fft_plane<64,0,1> 2,109,952 bytes read
# and no DRAM writes (the 2 MB grid's writes stay in L2 within a launch).
# Keyed by (kernel, workload, transform); null elsewhere.
MEASURED_TRAFFIC = {("fft_conv", "water12288", "own"): 7380480}


def measured_traffic(kernel, workload, fft):
    path = "own" if fft in ("auto", "own") else fft
    v = MEASURED_TRAFFIC.get((kernel, workload, path))
    return (v, "ncu capture of the same kernels on this workload") if v is not None else (None, None)


def oracle_solves(s, tr, first, nhist, ntimed, budget_s=None):
    """FP64 oracle solves on frames first-nhist .. first+ntimed-1 of the
    trajectory: nhist untimed solves fill the 16-frame ASPC history (started
    from alpha E), then up to ntimed timed solves start from the ASPC
    extrapolation, as the GPU arm's do.  budget_s bounds the timed part.
    Returns (seconds per timed solve list, iterations list)."""
    from oracle import oracle as O

    n3 = 3 * s.n
    hd, hp = np.zeros((16, n3)), np.zeros((16, n3))
    nualt = 0
    times, iters = [], []
    t_start = time.perf_counter()
    for k in range(nhist + ntimed):
        x = tr.frame(first - nhist + k)
        t0 = time.perf_counter()
        o = O.OracleSystem(s, xyz=x)
        if nualt >= 16:
            u0 = O.aspc_sum(hd, nualt).reshape(s.n, 3)
            p0 = O.aspc_sum(hp, nualt).reshape(s.n, 3)
            u = o.induce(uind0=u0, uinp0=p0)
        else:
            u = o.induce()
        dt = time.perf_counter() - t0
        hd[nualt % 16], hp[nualt % 16] = u[0].reshape(-1), u[1].reshape(-1)
        nualt += 1
        if k >= nhist:
            times.append(dt)
            iters.append(u[4])
            if budget_s is not None and time.perf_counter() - t_start > budget_s and len(times) >= 1:
                break
    return times, iters


def run_reference(args, world, rank):
    """CPU implementation of the step (oracle port, all host threads): the
    same frames and the same ASPC start as the GPU arm."""
    if rank != 0:
        return
    tg = importlib.import_module("tinker-gpu_gb300")
    from oracle import oracle as O

    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    s = tg.systems.make_config(args.config)
    tr = tg.systems.Trajectory(s)
    nhist = 16 if args.predictor == "aspc" else 0
    first = args.history + args.warmup
    times, iters = oracle_solves(s, tr, first, nhist, args.steps)
    sec = float(np.sum(times))
    value = len(times) / sec
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "induce() calls/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000 * sec / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded AMOEBA water trajectory)",
        "config": {"workload": args.config, "atoms": s.n, "pme_grid": list(s.settings["nfft"]),
                   "poleps_debye": s.settings["poleps"],
                   "guess": "ASPC over the 16 previous frames" if nhist else "direct (alpha E)"},
        "pcg_iterations_per_step": float(np.mean(iters)),
        "cpu_baseline": {"value": value, "unit": "induce() calls/s", "cores": cores, "kind": "port",
                         "sample": f"{len(times)} timed induce() calls on {args.config} (frames {first}.., FP64, "
                                   f"{'ASPC after ' + str(nhist) + ' untimed history solves' if nhist else 'direct guess'})"},
        "e2e": {"value": value, "unit": "induce() calls/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(args, s, tr):
    """One bounded sample of the CPU implementation (oracle port, all host
    threads): 16 untimed history solves, then ASPC-started solves for about
    20 s."""
    from oracle import oracle as O

    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    nhist = 16 if args.predictor == "aspc" else 0
    times, iters = oracle_solves(s, tr, args.history, nhist, 64, budget_s=20.0)
    return {"value": len(times) / float(np.sum(times)), "unit": "induce() calls/s", "cores": cores, "kind": "port",
            "sample": f"{len(times)} induce() calls on {args.config} (FP64, all host threads, "
                      f"{'ASPC after ' + str(nhist) + ' untimed history solves' if nhist else 'direct guess'}), "
                      f"{float(np.mean(iters)):.1f} iterations each"}


def kernel_rooflines(kernels, n, entries, nfft, peak):
    """Algorithmic bytes per launch / average event time of each profiled kernel."""
    out = {}
    for k, v in kernels.items():
        if not v.get("ms_per_launch"):
            continue
        alg = algorithmic_bytes(k, n, entries, nfft)
        gbs = alg / (v["ms_per_launch"] / 1000.0) / 1e9
        out[k] = {"algorithmic_bytes": alg, "achieved_gbs": gbs, "frac": gbs / peak}
    return out


# ring frames of the learned extrapolation (t9gb_learn_extrapolation) in its legs
LX_ORDER = 8


def lx_state(eng):
    """Fits, rejected fits and the fitted ring coefficients (newest frame
    first) of an engine's learned extrapolation."""
    fits, rej, cf = eng.learn_extrapolation_state()
    return {"fits": fits, "rejected_fits": rej, "ring_coefficients": [round(float(c), 5) for c in cf[:LX_ORDER]]}


def md_leg(args, abi, tg, stream, nrec, local, config, lx=0):
    """ns/day: velocity-Verlet MD of the configuration with the whole water
    force field -- multipole + polarization (induce with the ASPC predictor,
    PCG to 1e-6 D), buffered 14-7 van der Waals (9 A, taper from 8.1 A) and
    the water bond / angle / Urey-Bradley terms -- under the Bussi thermostat
    at 298 K, 1 fs steps.  From seeded Maxwell-Boltzmann velocities on the
    synthetic lattice: 2 ps of untimed NVT relaxation (the first 0.2 ps at a
    tau of 0.01 ps, while the randomly oriented waters release their packing
    energy as heat, then tau 0.1 ps), --md-steps timed steps, then nrec more
    steps recorded frame by frame on the device for the induce legs.
    Returns (result, recorded frames [nrec][n][3] float32 or None, system)."""
    import torch

    s = tg.systems.make_config(config, vdw=True, valence=True)
    mass = np.where(s.types == tg.systems.WATER_O, 15.999,
                    np.where(s.types == tg.systems.WATER_H, 1.008,
                             np.where(s.types == tg.systems.NA_ION, 22.99, 35.453)))
    rng = np.random.default_rng(29)
    v0 = rng.normal(size=(s.n, 3)) * np.sqrt(1.987204259e-3 * 298.0 * 418.4 / mass)[:, None]
    eng = abi.Engine(s, predictor=1, stream=stream)
    eng.prepare(s.xyz)
    if args.fft != "auto":
        eng.pme_own_fft(args.fft == "own")
    if lx:
        eng.learn_extrapolation(lx)
    dt = 1e-3
    K = args.md_steps
    eng.md_init(s.xyz, mass, v0)

    bad = []

    def run(n, tau):
        ek, t, rc = eng.md_run(n, dt, thermostat=1, kelvin=298.0, tau_ps=tau, seed=3)
        if rc != 0:
            bad.append(rc)
        return ek, t, rc

    with torch.cuda.stream(stream):
        run(200, 0.01)
        _, t_relax, _ = run(1800, 0.1)
        run(max(args.warmup, 3), 0.1)
        st0, it0 = eng.md_stats()
        clocks = ClockSampler(local)
        clocks.start()
        time.sleep(0.3)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        a.record(stream)
        ek, temp, _ = run(K, 0.1)
        b.record(stream)
        b.synchronize()
        wall = time.perf_counter() - w0
        ck = clocks.stop()
        st1, it1 = eng.md_stats()
        frames = None
        if nrec > 0:
            frames = torch.empty((nrec, s.n, 3), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            for k in range(nrec):
                run(1, 0.1)
                eng.md_positions_device(frames[k])
            torch.cuda.synchronize()
    ms = a.elapsed_time(b) / K
    lxs = lx_state(eng) if lx else None
    eng.close()
    return {
        "ms_per_step": ms,
        "wall_ms_per_step": 1000 * wall / K,
        "ns_per_day": 86.4 * dt * 1000 / ms,
        "steps": K,
        "pcg_iterations_per_step": (it1 - it0) / max(1, st1 - st0),
        "temperature_k": temp,
        "relaxation": {"ps": 2.0, "temperature_k": t_relax,
                       "schedule": "0.2 ps Bussi tau 0.01 ps, 1.8 ps Bussi tau 0.1 ps, 298 K"},
        "clocks": ck,
        "recorded_frames": nrec,
        **({"extrapolation": lxs} if lxs else {}),
        "status": "ok" if not bad else f"solver status {bad[0]} in {len(bad)} run(s): trajectory stopped early",
        "config": f"{config}: {s.n} atoms, PME {s.settings['nfft'][0]}^3; multipole + polarization (ASPC, PCG "
                  "1e-6 D), HAL 9 A, water valence; Bussi 298 K (tau 0.1 ps), 1 fs velocity Verlet",
    }, frames, s


def md_frames_leg(args, abi, s, stream, frames, flush, lx=0):
    """induce() ms/step and PCG iterations on frames of the relaxed box's MD
    trajectory (recorded by the MD leg): the configured workload's
    coordinates, rougher than the synthetic librating trajectory of `value`.
    ASPC after --history frames, --warmup untimed, --steps timed."""
    import torch

    H, W, K = args.history, args.warmup, args.steps
    if frames is None or frames.shape[0] < H + W + K:
        return None
    eng = abi.Engine(s, predictor=1 if args.predictor == "aspc" else 0, stream=stream)
    eng.prepare(frames[0].double().cpu().numpy())
    if lx:
        eng.learn_extrapolation(lx)
    ud = torch.zeros((s.n, 3), device="cuda")
    up = torch.zeros((s.n, 3), device="cuda")
    time_steps(eng, frames, range(H + W), stream, flush, ud, up)
    ms, its, _ = time_steps(eng, frames, range(H + W, H + W + K), stream, flush, ud, up)
    lxs = lx_state(eng) if lx else None
    eng.close()
    out = {"induce_ms_per_step": float(np.mean(ms)), "pcg_iterations_per_step": float(np.mean(its)),
           "steps": K, "frames": "MD trajectory of the relaxed box (2 ps NVT, then the timed MD steps)"}
    if lx:
        out["start"] = f"learned extrapolation of the ASPC ring ({lx} frames, fitted online)"
        out["extrapolation"] = lxs
    return out


def large_leg(args, abi, tg, stream, flush, peak):
    """The 98,304-atom box (PME 128^3): induce ms/step in the graph, per-kernel
    rooflines from a profiled pass, and the learned-guess legs."""
    import torch

    s = tg.systems.make_config(args.large_config)
    tr = tg.systems.Trajectory(s, seed=17)
    eng = abi.Engine(s, predictor=1, stream=stream)
    eng.prepare(tr.frame(0))
    if args.fft != "auto":
        eng.pme_own_fft(args.fft == "own")
    K, W, H = args.steps, args.warmup, args.history
    dev = torch.from_numpy(np.stack([tr.frame(t) for t in range(H + W + 2 * K)]).astype(np.float32)).to("cuda")
    ud = torch.zeros((s.n, 3), device="cuda")
    up = torch.zeros((s.n, 3), device="cuda")
    time_steps(eng, dev, range(H + W), stream, flush, ud, up)
    ms, its, _ = time_steps(eng, dev, range(H + W, H + W + K), stream, flush, ud, up)
    eng.profile(True)
    eng.profile_read(reset=True)
    with torch.cuda.stream(stream):
        for t in range(H + W + K, H + W + 2 * K):
            eng.set_xyz_device(dev[t])
            eng.mpole_init()
            eng.induce(out=(ud, up))
    prof = eng.profile_read(reset=True)
    eng.profile(False)
    kernels = {k: {"ms_total": v[0], "launches": v[1], "ms_per_launch": (v[0] / v[1] if v[1] else None)}
               for k, v in prof.items() if v[1]}
    ls = eng.list_stats()
    e2 = abi.Engine(s, predictor=1, stream=stream)
    e2.prepare(tr.frame(0))
    if args.fft != "auto":
        e2.pme_own_fft(args.fft == "own")
    e2.learn_extrapolation(LX_ORDER)
    time_steps(e2, dev, range(H + W), stream, flush, ud, up)
    lms, lits, _ = time_steps(e2, dev, range(H + W, H + W + K), stream, flush, ud, up)
    lxs = lx_state(e2)
    e2.close()
    out = {"workload": args.large_config, "atoms": s.n, "pme_grid": list(s.settings["nfft"]),
           "induce_ms_per_step": float(np.mean(ms)), "pcg_iterations_per_step": float(np.mean(its)),
           "induce_learned_extrapolation": {"induce_ms_per_step": float(np.mean(lms)),
                                            "pcg_iterations_per_step": float(np.mean(lits)),
                                            "speedup_vs_aspc": float(np.mean(ms)) / float(np.mean(lms)),
                                            "extrapolation": lxs},
           "kernels": kernels,
           "rooflines": kernel_rooflines(kernels, s.n, ls["entries"], s.settings["nfft"][0], peak)}
    eng.close()
    if not args.no_learned and args.learn_train > 0:
        nfr = args.learn_train + 4 * (args.warmup + args.steps)
        x0 = 100000  # frames after the measurement's
        lf = torch.from_numpy(np.stack([tr.frame(x0 + t) for t in range(nfr)]).astype(np.float32)).to("cuda")
        out["learned_guess"] = learned_legs(args, s, abi, stream, lf, flush, check_oracle=False)
        out["learned_guess"]["frames"] = "synthetic librating trajectory"
    return out


def time_steps(eng, dev_frames, idxs, stream, flush, ud, up):
    """CUDA-event time of induce() on the given device frames (L2 flushed
    before each step, outside the brackets); returns (ms list, iterations,
    learned-guess stats)."""
    import torch

    ms, its, ls = [], [], []
    with torch.cuda.stream(stream):
        for k, t in enumerate(idxs):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.set_xyz_device(dev_frames[t])
            eng.mpole_init()
            eng.induce(out=(ud, up))
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
            its.append(eng.stats()[0])
            ls.append(eng.learn_stats())
    return ms, its, ls


def learned_legs(args, s, abi, stream, dev, flush, check_oracle, timed=None):
    """The learned initial guess against the plain guesses.

    Two engines follow the trajectory: one with the direct guess alpha E (no
    predictor), one with the ASPC predictor.  Each trains its network online
    for --learn-train steps (one AdamW step per solve on its converged
    dipoles, plain starts), then continues the trajectory through three timed
    legs of --steps frames, each after --warmup untimed frames: the plain
    start (network off), the learned start compared with the plain one on
    every solve (probe 1), and the comparison on every 16th solve (probe 16).
    Training is off in the timed legs.  The ASPC engine adds a fourth leg: the
    learned extrapolation of its ring (LX_ORDER frames, fitted online after
    every solve).  dev: device frames [>= T + 4 (W + K)][n][3];
    K = timed (default --steps)."""
    import torch

    T, K, W = args.learn_train, timed or args.steps, args.warmup
    assert dev.shape[0] >= T + 4 * (W + K)
    ud = torch.zeros((s.n, 3), device="cuda")
    up = torch.zeros((s.n, 3), device="cuda")
    out = {"train_steps": T, "timed_steps": K, "rows_per_batch": 2 * s.n,
           "network": "32-64-64-3 SiLU, BF16 weights/activations, FP32 accumulation, AdamW lr 1e-3 wd 1e-2"}
    for pred, name in ((0, "direct"), (1, "aspc")):
        eng = abi.Engine(s, predictor=pred, stream=stream)
        eng.prepare(dev[0].double().cpu().numpy())
        if args.stepwise:
            eng.use_graph(False)
        eng.learn_reset(seed=1)
        eng.learn_config(1)
        t0 = time.perf_counter()
        tr_ms, tr_it, tr_ls = time_steps(eng, dev, range(T), stream, flush, ud, up)
        res = {"train_ms_per_step": float(np.mean(tr_ms[-50:])), "train_iters_last50": float(np.mean(tr_it[-50:])),
               "train_loss_last": tr_ls[-1][3], "train_wall_s": time.perf_counter() - t0}
        f = T
        legs = [(0, 1, "plain"), (2, 1, "learned_probe1"), (2, 16, "learned_probe16")]
        if pred == 1:
            legs.append((0, 1, "learned_extrapolation"))
        for mode, probe, leg in legs:
            eng.learn_config(mode)
            eng.learn_policy(probe)
            if leg == "learned_extrapolation":
                eng.learn_extrapolation(LX_ORDER)
            time_steps(eng, dev, range(f, f + W), stream, flush, ud, up)
            idx = list(range(f + W, f + W + K))
            f += W + K
            ms, its, ls = time_steps(eng, dev, idx, stream, flush, ud, up)
            r = {"induce_ms_per_step": float(np.mean(ms)), "pcg_iterations_per_step": float(np.mean(its))}
            if leg == "learned_extrapolation":
                r["extrapolation"] = lx_state(eng)
                r["iterations_histogram"] = np.bincount(its).tolist()
            if mode == 2:
                r["learned_start_fraction"] = float(np.mean([((c & 1) + ((c >> 1) & 1)) / 2 for c, *_ in ls]))
                r["compared_fraction"] = float(np.mean([l[4] for l in ls]))
                cmp_ = [l for l in ls if l[4]]
                r["start_residual_plain_debye"] = float(np.mean([l[1] for l in cmp_])) if cmp_ else None
                r["start_residual_learned_debye"] = float(np.mean([l[2] for l in cmp_])) if cmp_ else None
                if check_oracle and probe == 1:
                    from oracle import oracle as O

                    xyz = dev[idx[-1]].double().cpu().numpy()
                    ou, op, *_ = O.OracleSystem(s, xyz=xyz).induce()
                    D = importlib.import_module("tinker-gpu_gb300.units").DEBYE
                    g_ud = ud.double().cpu().numpy()
                    g_up = up.double().cpu().numpy()
                    r["oracle_rms_dipole_error_debye"] = float(max(
                        np.sqrt(((g_ud - ou) ** 2).sum(1).mean()) * D, np.sqrt(((g_up - op) ** 2).sum(1).mean()) * D))
            res[leg] = r
        for leg in ("learned_probe1", "learned_probe16", "learned_extrapolation"):
            if leg in res:
                res[leg]["speedup_vs_plain"] = res["plain"]["induce_ms_per_step"] / res[leg]["induce_ms_per_step"]
        out[name] = res
        eng.close()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
        run_reference(args, world, rank)
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    tg = importlib.import_module("tinker-gpu_gb300")
    b = importlib.import_module("tinker-gpu_gb300.build")
    b.build()
    abi = importlib.import_module("tinker-gpu_gb300.abi")

    s = tg.systems.make_config(args.config)
    tr = tg.systems.Trajectory(s, seed=11 + rank)
    pred = 1 if args.predictor == "aspc" else 0
    stream = torch.cuda.Stream()
    eng = abi.Engine(s, predictor=pred, stream=stream)
    eng.prepare(tr.frame(0))
    if args.fft != "auto":
        eng.pme_own_fft(args.fft == "own")
    if args.lanes:
        eng.pair_lanes(args.lanes)
    # frames: predictor history, warm-up, then the timed, e2e, per-kernel and
    # force passes, each continuing the trajectory (no time jumps for the predictor)
    f0 = args.history + args.warmup
    nsteps = f0 + 4 * args.steps
    frames = np.stack([tr.frame(t) for t in range(nsteps)]).astype(np.float32)
    # device-resident inputs for the kernel-only measurement
    dev_frames = torch.from_numpy(frames).to("cuda")
    ud = torch.zeros((s.n, 3), device="cuda")
    up = torch.zeros((s.n, 3), device="cuda")
    flush = torch.empty((16 if args.no_flush else 512 * 1024 * 1024) // 4, dtype=torch.float32, device="cuda")

    def step_device(t):
        eng.set_xyz_device(dev_frames[t])
        eng.mpole_init()
        eng.induce(out=(ud, up))

    # trajectory history fills the predictor ring (outside every timed region)
    with torch.cuda.stream(stream):
        for t in range(args.history):
            step_device(t)
        for t in range(args.history, args.history + args.warmup):
            step_device(t)
    torch.cuda.synchronize()

    # ---- timed region: device-resident inputs ----
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    iters = []
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            step_device(args.history + args.warmup + k)
            ev[k][1].record(stream)
            iters.append(eng.stats()[0])
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        dist.barrier()
    ck = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_sec = sum(step_ms) / 1000.0
    if world > 1:
        t = torch.tensor([dev_sec], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_sec = float(t.item())
    value = world * args.steps / dev_sec

    # ---- the same frames from the learned extrapolation of the ASPC ring ----
    lx_res = None
    if pred == 1:
        e2 = abi.Engine(s, predictor=1, stream=stream)
        e2.prepare(tr.frame(0))
        if args.fft != "auto":
            e2.pme_own_fft(args.fft == "own")
        if args.lanes:
            e2.pair_lanes(args.lanes)
        e2.learn_extrapolation(LX_ORDER)
        time_steps(e2, dev_frames, range(args.history + args.warmup), stream, flush, ud, up)
        lms, lits, _ = time_steps(e2, dev_frames, range(args.history + args.warmup,
                                                         args.history + args.warmup + args.steps), stream, flush, ud, up)
        lxs = lx_state(e2)
        e2.close()
        lx_res = {"induce_ms_per_step": float(np.mean(lms)), "pcg_iterations_per_step": float(np.mean(lits)),
                  "speedup_vs_aspc": (1000 * dev_sec / args.steps) / float(np.mean(lms)),
                  "start": f"learned extrapolation of the ASPC ring ({LX_ORDER} frames, fitted online after every "
                           "solve)", "frames": "the timed frames of value", "extrapolation": lxs}

    # ---- e2e: host coordinates in, host dipoles out ----
    hu = np.zeros((s.n, 3))
    hp = np.zeros((s.n, 3))
    e2e_t = []
    for k in range(args.steps):
        x = frames[f0 + args.steps + k].astype(np.float64)
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.induce_host(x, hu, hp)
        e2e_t.append(time.perf_counter() - t0)
    e2e_sec = float(np.sum(e2e_t))
    if world > 1:
        t = torch.tensor([e2e_sec], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_sec = float(t.item())
    e2e_value = world * args.steps / e2e_sec

    # ---- per-kernel timing pass (CUDA events on the library stream) ----
    eng.profile(True)
    eng.profile_read(reset=True)
    prof_iters = []
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            step_device(f0 + 2 * args.steps + k)
            prof_iters.append(eng.stats()[0])
    prof = eng.profile_read(reset=True)
    eng.profile(False)
    kernels = {k: {"ms_total": v[0], "launches": v[1], "ms_per_launch": (v[0] / v[1] if v[1] else None)}
               for k, v in prof.items() if v[1]}
    dom = max(kernels, key=lambda k: kernels[k]["ms_total"])
    traffic, traffic_src = measured_traffic(dom, args.config, args.fft)
    nfft = s.settings["nfft"][0]
    ls = eng.list_stats()
    alg = algorithmic_bytes(dom, s.n, ls["entries"], nfft)
    peak, peak_kind = measured_peaks()
    per_launch_s = kernels[dom]["ms_per_launch"] / 1000.0
    achieved = alg / per_launch_s / 1e9
    mean_it = float(np.mean(iters))
    # own kernels per step (fused FFT, default CG fusion; programmatic launches count as launches): positions 1, rotpole 2, list 5, permanent
    # field 6 (real, spread, 3 transform, gather), guess 1, field of the guess 6, r0 1, M r0 with the
    # dots 1, peek + predictor save 1, predictor index 1, output 1; per PCG iteration: direction 1,
    # field 6, Ap 1, update 1, M r with the dots 1
    launches_per_step = 26 + 10 * mean_it

    # ---- forces: emplar (induce + multipole and polarization energy, gradient, virial) ----
    forces = None
    if not args.no_forces:
        fms = []
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                eng.set_xyz_device(dev_frames[f0 + 3 * args.steps + k])
                eng.mpole_init()
                flush.fill_(float(k))
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                eng.emplar(abi.CALC_ENERGY | abi.CALC_GRAD | abi.CALC_VIRIAL)
                b.record(stream)
                b.synchronize()
                fms.append(a.elapsed_time(b))
        em = float(np.mean(fms))
        forces = {"emplar_ms_per_step": em, "induce_ms_per_step": 1000 * dev_sec / args.steps,
                  "forces_virial_ms_per_step": em - 1000 * dev_sec / args.steps,
                  "note": "t9gb_emplar(energy|grad|virial): induce + real-space and PME forces, torques, virial"}

    # ---- MD (ns/day), recording the frames of the learned-guess legs ----
    want_learned = not args.no_learned and args.learn_train > 0
    nrec = args.learn_train + 4 * (args.warmup + args.learn_steps) if want_learned else 0
    nrec = max(nrec, args.history + args.warmup + args.steps)
    md, md_frames, md_sys = None, None, None
    if not args.no_md:
        md, md_frames, md_sys = md_leg(args, abi, tg, stream, nrec, local, args.config)

    md_frames_res = md_frames_lx = None
    if md_frames is not None:
        md_frames_res = md_frames_leg(args, abi, md_sys, stream, md_frames, flush)
        if pred == 1:
            md_frames_lx = md_frames_leg(args, abi, md_sys, stream, md_frames, flush, lx=LX_ORDER)
            md_frames_lx["speedup_vs_aspc"] = md_frames_res["induce_ms_per_step"] / md_frames_lx["induce_ms_per_step"]

    learned = None
    if want_learned:
        check = rank == 0 and not args.no_cpu_baseline
        if md_frames is not None:
            learned = learned_legs(args, md_sys, abi, stream, md_frames, flush, check_oracle=check,
                                   timed=args.learn_steps)
            learned["frames"] = "MD trajectory of the relaxed box (the MD leg's, continued)"
        else:
            lf = torch.from_numpy(np.stack([tr.frame(100000 + t) for t in range(nrec)]).astype(np.float32)).to("cuda")
            learned = learned_legs(args, s, abi, stream, lf, flush, check_oracle=check, timed=args.learn_steps)
            learned["frames"] = "synthetic librating trajectory"
        del md_frames

    large = None
    if not args.no_large:
        large = large_leg(args, abi, tg, stream, flush, peak)

    # ---- MD of the other configurations (ns/day only), and of this one from
    # the learned extrapolation of the ASPC ring ----
    md_other = {}
    md_lx = None
    if not args.no_md:
        for name in [c for c in args.md_extra.split(",") if c and c != args.config]:
            md_other[name] = md_leg(args, abi, tg, stream, 0, local, name)[0]
        md_lx = md_leg(args, abi, tg, stream, 0, local, args.config, lx=LX_ORDER)[0]
        md_lx["start"] = f"learned extrapolation of the ASPC ring ({LX_ORDER} frames, fitted online after every solve)"

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(args, s, tr)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "induce() calls/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": 1000 * dev_sec / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 pair/spline math, fixed-point i64 accumulation, f64 PCG scalars",
            "data": "synthetic (seeded AMOEBA water lattice, 1 fs librating trajectory)",
            "config": {
                "workload": args.config, "atoms": s.n, "pme_grid": list(s.settings["nfft"]), "cutoff_A": 7.0,
                "poleps_debye": s.settings["poleps"], "predictor": args.predictor, "history_frames": args.history,
                "fft": {"auto": "library default: fused transform on cubic 32/64 grids, cuFFT C2C otherwise",
                        "own": "fused power-of-two transform (library)", "cufft": "cuFFT C2C"}[args.fft],
                "lanes_per_atom": args.lanes or "library default (8 up to 32,768 atoms, 4 above)",
                "l2": "not flushed (profiling run)" if args.no_flush else "flushed (512 MB write) between timed steps",
                "parallelism": f"replicas x{world}",
            },
            "induce_ms_per_step": 1000 * dev_sec / args.steps,
            "pcg_iterations_per_step": mean_it,
            "induce_md_frames": md_frames_res,
            "induce_learned_extrapolation": lx_res,
            "induce_md_frames_learned_extrapolation": md_frames_lx,
            "induce_note": "value and induce_ms_per_step: the seeded librating trajectory (smoother than MD: "
                           "fewer PCG iterations), ASPC start as the reference; induce_md_frames: the same solve "
                           "on frames of the relaxed box's MD trajectory; *_learned_extrapolation: the same frames "
                           "from the learned extrapolation of the ASPC ring",
            "ns_per_day": None if md is None else md["ns_per_day"],
            "ns_per_day_note": "MD leg (see md)" if md is not None else "MD leg skipped (--no-md)",
            "md": md,
            "md_learned_extrapolation": md_lx,
            "md_other_configs": md_other,
            "wall_s_timed": wall,
            "e2e": {"value": e2e_value, "unit": "induce() calls/s", "ms_per_step": 1000 * e2e_sec / args.steps,
                    "h2d_bytes_per_step": 3 * s.n * 4, "d2h_bytes_per_step": 6 * s.n * 4},
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": alg,
                         "algorithmic_basis": "compulsory bytes per launch (see algorithmic_bytes in bench.py)",
                         "transform_pass_bytes_per_launch": (FFT_PASS_BYTES * nfft ** 3 if dom == "fft_conv"
                                                             else None)},
            "kernels": kernels,
            "kernel_rooflines": kernel_rooflines(kernels, s.n, ls["entries"], nfft, peak),
            "lists": ls,
            "gpu_launches": int(round(launches_per_step * args.steps)),
            "clocks": ck,
            "cpu_baseline": cpu,
            "learned_guess": learned,
            "forces": forces,
            "large_box": large,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
