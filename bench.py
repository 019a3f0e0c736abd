"""Throughput of the short-range particle step on one GB300 (particle-steps/s).

Workload (the ~10^6-bead membrane system the metric is quoted on):
  membrane_1m - 10 flat bilayers of 1-hydrophilic + 3-hydrophobic chains
  stacked along z in a periodic 64 x 64 x 48 box, area per lipid 0.333
  (input_generator.py:69), 246,010 molecules = 984,040 beads; reference MDPD
  form (chi 30, kappa 100, rho_co 40, vbb 0.1), sigma 3, dt 0.005, bonds
  cf_s = 50 (k = cf_s / l0 = 100, l0 = 0.5), bend cf_b = 10. Seeded synthetic
  input (no dataset is involved).

Arms:
  engine (default)  the FP32-pair / fixed-point engine, one CUDA graph per step;
                    also reports the plain FP64 pair kernels on the same
                    workload, the end-to-end rate through the C ABI with pinned
                    host buffers, the roofline of the force kernel and the CPU
                    oracle on a bounded sample (cpu_baseline).
  reference         the reference's CPU algorithm (the C oracle, all host
                    threads) on a bounded sample of the same workload.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from implicit_dpd_gb300 import configs  # noqa: E402

BOX = np.array([64.0, 64.0, 48.0])
N_LAYERS = 10
AREA_PER_LIPID = 0.333
METRIC = "particle-steps/s on 1 GB300: FP32+batched vs plain FP64 kernel at stated force err"
# Algorithmic HBM bytes per particle of the two pair passes: the density pass
# reads the particle's posf (16 B) and writes its densf (16 B); the force pass
# reads posf, velf, densf (3 x 16 B) and writes the fixed-point force (3 x 8 B).
PAIR_KERNELS = {
    "density": {"kernel": "k_density_f32", "bytes_per_particle": 32,
                "profile": "density_membrane_1m.md"},
    "force": {"kernel": "k_force_f32", "bytes_per_particle": 72,
              "profile": "force_membrane_1m.md"},
}
STEP_BYTES_PER_PARTICLE = 176  # compulsory HBM bytes of one particle-step
# Algorithmic lane operations per in-range ordered pair (the reference
# evaluates every pair from both sides): the force pass ~54 FP32 + ~75 INT32
# (the Saru hash and draws) + 5 SFU (sqrt r, rcp, sqrt w, log, cos); the
# density pass ~12 FP32 + 1 SFU.
OPS_PER_ORDERED_PAIR = {"force": 134, "density": 13}
# Kernels a captured step launches (the loop node repeats them): without kept
# lists drift_bin, scan x3, scatter, cell_sort, pack, density, density
# finalize, force, force walk, bonded_kick, the drift-removal condition, time,
# the loop's tail; with kept lists drift_disp, rebuild decision, two rebuild
# conditions, pack, density (kept lists, overflowed kept lists), density
# finalize, force, force walk, bonded_kick, the drift-removal condition, time,
# the loop's tail. A rebuild step adds the IF body of the cells and lists (bin,
# scan x3, scatter, cell_sort, list build); a step whose replica counter is a
# multiple of 100 adds the drift removal (3 kernels).
KERNELS_PER_STEP = 15
KERNELS_PER_KEPT_STEP = 14
KERNELS_PER_REBUILD = 7
KERNELS_PER_CM = 3
KERNELS_PER_REORDER = 4        # gather, topology, identity, loc


def n_amp_for(box, layers):
    return layers * int(round(2 * box[0] * box[1] / AREA_PER_LIPID))


def workload(box=BOX, layers=N_LAYERS, seed=20250101):
    n_amp = n_amp_for(box, layers)
    st = configs.flat_bilayers(box, n_amp, seed=seed, n_layers=layers)
    rp = configs.run_param(box, dt=0.005, cf_r=3.0, cf_s=50.0, cf_b=10.0, vbb=0.1, chi=30.0,
                           kappa=100.0, rho_co=40.0)
    return st, n_amp, rp


def workload_name(box=BOX, layers=N_LAYERS):
    box = np.asarray(box, np.float64)
    if np.array_equal(box, BOX) and layers == N_LAYERS:
        return "membrane_1m"
    return "membrane_{:g}x{:g}x{:g}_{}layers".format(*box, layers)


def workload_desc(n, n_amp, box=BOX, layers=N_LAYERS):
    return {
        "workload": workload_name(box, layers),
        "description": (f"{layers} flat bilayers of 1H+3T chains stacked in a periodic "
                        "{:g}x{:g}x{:g} box, ".format(*box) +
                        "reference MDPD form (chi 30, kappa 100, rho_co 40, vbb 0.1), sigma 3, "
                        "dt 0.005, cf_s 50, cf_b 10; timed after the equilibration steps, when "
                        "the bilayers have compacted to ~150 ordered pairs within the cutoff per "
                        "bead"),
        "n_particles": int(n),
        "n_molecules": int(n_amp),
        "l2": ("inputs larger than L2: the pair passes read posf, poslo, velf, densf and the "
               f"neighbour list, ~{n * 344 / 1e6:.0f} MB per step against a 129 MB L2"),
    }


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


class Dist:
    def __init__(self, world):
        self.pg = None
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td
            self.pg = True

    def barrier(self):
        if self.pg:
            self.td.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def gather(self, obj):
        """Every rank's obj, in rank order (host objects over gloo)."""
        if not self.pg:
            return [obj]
        out = [None] * self.td.get_world_size()
        self.td.all_gather_object(out, obj)
        return out

    def close(self):
        if self.pg:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        """Starts sampling every 20 ms and returns once the first sample is
        written (nvidia-smi takes ~0.1 s to start), so that even a timed region
        of a few tens of ms falls inside the sampled window."""
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.005)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]) if f[3] not in ("[N/A]", "N/A") else 0.0,
                             f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "reasons": reasons, "samples": len(rows)}


def cpu_info():
    """CPU model of the host and the thread settings the CPU arms use."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                model = line.split(":", 1)[1].strip()
                if not model.isdigit():
                    break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"cpu_model": model, "nproc": os.cpu_count(),
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS"),
            "threads_used": os.cpu_count() or 1,
            "threads_note": "the oracle's OpenMP loops run os.cpu_count() threads (num_threads "
                            "passed explicitly; OMP_NUM_THREADS is not read)"}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(name):
    """DRAM bytes per launch of a kernel from its committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def equilibrated_patch(threads, equil=2000):
    """An 8 x 8 x 48 periodic column of membrane_1m (the same ten stacked
    bilayers and box height, 15,360 beads) taken through `equil` oracle steps:
    the compaction the timed GPU state went through, so the CPU sample has the
    GPU state's pairs per bead. Returns (state, patch box, molecules, params)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O

    small = np.array([8.0, 8.0, BOX[2]])
    st, n_amp, rp = workload(box=small, layers=N_LAYERS, seed=7)
    p = O.derive_params(rp)
    p.seed, p.time = 1, 1
    st["topol"], st["cf_bend"] = O.build_topology(st["amp_id"], st["unit"], n_amp, [], p.cf_b,
                                                  p.cf_b_rigid)
    for _ in range(equil):
        O.md_step(p, st, nthreads=threads)
    st["pos"] -= np.floor(st["pos"] / small) * small
    return st, small, n_amp, p


def tile_patch(patch, reps):
    """reps = (nx, ny) periodic copies of the equilibrated column side by side:
    a (8 nx) x (8 ny) x 48 section of membrane_1m."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O

    st, small, n_amp, p = patch
    big, box = configs.tile({k: st[k] for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")},
                            small, (reps[0], reps[1], 1))
    n_amp_big = n_amp * reps[0] * reps[1]
    rp_big = configs.run_param(box, dt=0.005, cf_r=3.0, cf_s=50.0, cf_b=10.0, vbb=0.1, chi=30.0,
                               kappa=100.0, rho_co=40.0)
    pb = O.derive_params(rp_big)
    pb.seed, pb.time = 1, p.time
    big["topol"], big["cf_bend"] = O.build_topology(big["amp_id"], big["unit"], n_amp_big, [],
                                                    pb.cf_b, pb.cf_b_rigid)
    return big, n_amp_big, pb, box


def cpu_baseline(state, n_amp, rp, time_step, min_seconds=10.0, max_steps=50):
    """The C oracle (the reference's CPU algorithm, FP64) timed on the GPU's own
    timed state (the whole workload, downloaded after the timed steps: the same
    configuration and pairs per bead as the GPU's figure), every host thread,
    for about min_seconds, with the parity build and with the reference's
    production flags."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O

    threads = os.cpu_count() or 1
    p = O.derive_params(rp)
    p.seed, p.time = 12345, int(time_step)
    st = {k: np.array(state[k], copy=True) for k in ("pos", "vel", "acc", "id", "prop")}
    st["topol"], st["cf_bend"] = O.build_topology(state["amp_id"], state["unit"], n_amp, [],
                                                  p.cf_b, p.cf_b_rigid)
    n = len(st["pos"])
    pairs = O.pair_count(p, st["pos"], threads) / n

    def timed(fast):
        O.use_fast_build(fast)
        try:
            O.md_step(p, st, nthreads=threads)  # warm-up
            steps = 0
            t0 = time.perf_counter()
            while steps < max_steps:
                O.md_step(p, st, nthreads=threads)
                steps += 1
                if time.perf_counter() - t0 >= min_seconds:
                    break
            return steps, time.perf_counter() - t0
        finally:
            O.use_fast_build(False)

    steps, dt = timed(False)
    steps_f, dt_f = timed(True)
    out = {"value": n * steps / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
           "sample": f"{steps} MD steps (drift, density, force, bonded, kick) of the GPU's timed "
                     f"state itself ({n} beads, {pairs:.1f} ordered pairs within the cutoff per "
                     f"bead), FP64 C oracle (-O2, no contraction), OpenMP",
           "pairs_per_bead": pairs,
           "production_flags": {"value": n * steps_f / dt_f, "unit": "particle-steps/s",
                                "steps": steps_f,
                                "flags": "-O3 -ffast-math -funroll-loops (the reference's "
                                         "Makefile:10,21-23)"}}
    out.update(cpu_info())
    return out


def run_reference(args, rank, world, budget_s=90.0):
    """The reference's CPU algorithm (the C oracle, every host thread) on a
    sample of the equilibrated membrane sized so that warm-up plus timed steps
    take about `budget_s` seconds."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O

    threads = os.cpu_count() or 1
    patch = equilibrated_patch(threads)
    # rate of the oracle on a 24 x 16 x 48 section, then the sample that fits the budget
    probe, _, pp, _ = tile_patch(patch, (3, 2))
    t0 = time.perf_counter()
    O.md_step(pp, probe, nthreads=threads)
    rate = len(probe["pos"]) / (time.perf_counter() - t0)
    per_step = budget_s / max(1, args.steps + args.warmup)
    tiles = int(min(64, max(1, rate * per_step // len(patch[0]["pos"]))))
    ny = min(8, tiles)
    nx = max(1, min(8, tiles // ny))
    st, n_amp, p, box = tile_patch(patch, (nx, ny))
    for _ in range(args.warmup):
        O.md_step(p, st, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.md_step(p, st, nthreads=threads)
    dt = time.perf_counter() - t0
    n = len(st["pos"])
    value = n * args.steps / dt
    pairs = O.pair_count(p, st["pos"], threads) / n
    sample = (f"each step one MD step (drift, density, force, bonded, kick) of an equilibrated "
              f"section of membrane_1m (the ten stacked bilayers, {box[0]:g}x{box[1]:g}x{box[2]:g}, {n} beads, "
              f"{pairs:.1f} ordered pairs within the cutoff per bead), FP64 C oracle of the "
              f"reference algorithm, OpenMP")
    out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic",
           "config": dict(workload_desc(n, n_amp),
                          sample=(f"a {nx} x {ny} lateral tiling of an 8 x 8 x 48 column of the "
                                  "same ten bilayers taken through 2,000 oracle steps (the GPU "
                                  "line times its own equilibrated 984,040-bead state; the "
                                  "per-bead rate of the CPU steps does not depend on the size)"),
                          pairs_per_bead=pairs),
           "impl": "reference",
           "cpu_baseline": dict({"value": value, "unit": "particle-steps/s", "cores": threads,
                                 "kind": "port", "sample": sample, "pairs_per_bead": pairs},
                                **cpu_info()),
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def reaction_bench(tune, steps=100, equil=2000, device=0):
    """The membrane with precursors: the stacked bilayers of the headline
    workload plus single precursor beads at 10% of the bead count, uniform in
    the box, each converted to a head bead with p = 1e-4 per step when a tail
    bead lies within the cutoff (Saru draw keyed on (id, step, seed)).
    Returns particle-steps/s with the conversion on, and the conversions."""
    from implicit_dpd_gb300.abi import HYPHIL, HYPHOB, SOLVENT, precursor_threshold

    st, n_amp, rp = workload()
    box = np.asarray(BOX, np.float64)
    n_pre = len(st["pos"]) // 10
    pre = configs.liquid(box, n_pre / box.prod(), seed=777, prop=SOLVENT)
    both = {k: np.concatenate([st[k], pre[k]]) for k in ("pos", "vel", "acc", "prop", "amp_id",
                                                          "unit")}
    n = len(both["pos"])
    both["id"] = np.arange(n, dtype=np.uint32)
    e = make_engine(both, n_amp, rp, device=device)
    e.set_tuning(tune["reach"], tune["skin"], lanes=tune.get("lanes"), blocks=tune.get("blocks"),
                 dens_lanes=tune.get("dens_lanes"))
    e.step(equil)
    e.set_precursor(SOLVENT, HYPHOB, HYPHIL, precursor_threshold(1e-4), 2024)
    e.step(3)
    e.sync()
    c0 = e.precursor_count()
    e.step(steps)
    ms = e.last_step_ms()
    conv = e.precursor_count() - c0
    e.close()
    return {"workload": "membrane_precursor_1m", "n_particles": int(n), "n_precursor": int(len(pre["pos"])),
            "steps": steps, "equilibration_steps": equil, "value": n * steps / (ms * 1e-3),
            "unit": "particle-steps/s", "ms_per_step": ms / steps, "conversions": int(conv),
            "tuning": tune,
            "description": "the membrane_1m bilayers plus 10% single precursor beads (uniform), "
                           "converted to heads with p = 1e-4 per step within the cutoff of a "
                           "tail bead (Saru(id, step, seed) draw, bit-exact decisions)"}


def liquid_workload():
    """The 10^6-particle MDPD liquid: 55^3 box at density 6 (998,250
    particles), Warren form A = -40, B = 25, r_d = 0.75, sigma 3, dt 0.005,
    uniform random start."""
    from implicit_dpd_gb300.abi import FORM_WARREN
    from implicit_dpd_gb300.engine import derive_params

    box = np.array([55.0, 55.0, 55.0])
    st = configs.liquid(box, 6.0, seed=12350)
    p = derive_params(configs.run_param(box, dt=0.005, cf_r=3.0))
    p.seed, p.time, p.form = 2468, 1, FORM_WARREN
    p.warren_a, p.warren_b, p.warren_rd = -40.0, 25.0, 0.75
    return box, st, p


# (reach, skin, lanes, blocks, pass-1 lanes) the package's tuner picks for the liquid
LIQUID_TUNE = (1, 0.3, 4, 2, 4)


def run_liquid_case(equil, device=0):
    """The liquid from its uniform start at its tuned shape: `equil` graph
    steps, then 12 more (kept-list steps, for launch lists of the liquid)."""
    from implicit_dpd_gb300.engine import Engine

    box, st, p = liquid_workload()
    e = Engine(flags=GRAPH_FLAGS, sort_period=100, device=device)
    e.set_params(p)
    e.upload(st)
    reach, skin, lanes, blocks, dl = LIQUID_TUNE
    e.set_tuning(reach, skin, lanes=lanes, blocks=blocks, dens_lanes=dl)
    e.step(equil)
    e.step(12)
    e.sync()
    print(json.dumps({"liquid_case": "mdpd_liquid_1m", "n_particles": len(st["pos"]),
                      "steps": equil + 12, "rebuilds": e.list_rebuilds(),
                      "tuning": dict(zip(("reach", "skin", "lanes", "blocks", "dens_lanes"),
                                         LIQUID_TUNE))}), flush=True)
    e.close()


def liquid_bench(steps=200, equil=300, device=0):
    """The 10^6-particle MDPD liquid (liquid_workload). The FP32 engine (tuned
    by the package's tuner) against the plain FP64 kernels of the same step,
    with the measured force error."""
    from implicit_dpd_gb300.abi import CFG_FP64_KEPT, CFG_FP64_PAIRS
    from implicit_dpd_gb300.engine import Engine

    box, st, p = liquid_workload()
    n = len(st["pos"])

    def engine(flags=0, state=st):
        e = Engine(flags=flags, sort_period=100, device=device)
        e.set_params(p)
        e.upload(state)
        return e

    e = engine()
    e.step(equil)
    # the package's tuner: (reach, skin), then the force pass's launch shape
    tuned, _ = autotune(e)
    reach, skin = tuned["reach"], tuned["skin"]
    e.step(3)
    e.step(steps)
    v32 = n * steps / (e.last_step_ms() * 1e-3)
    eq = e.download()
    e.close()
    st_eq = dict(st, pos=eq["pos"], vel=eq["vel"], acc=eq["acc"])
    e32, e64 = engine(state=st_eq), engine(CFG_FP64_PAIRS, st_eq)
    for x in (e32, e64):
        x.density()
        x.force()
    f32, f64 = e32.download()["acc"], e64.download()["acc"]
    e32.close()
    mag = np.linalg.norm(f64, axis=1)
    err = np.linalg.norm(f32 - f64, axis=1) / np.maximum(mag, np.sqrt(np.mean(mag ** 2)))
    e64.step(1)
    e64.step(10)
    v64 = n * 10 / (e64.last_step_ms() * 1e-3)
    e64.close()
    # the engine's own algorithm in FP64 (kept lists at reach 1, each pair once)
    ek = engine(CFG_FP64_KEPT, st_eq)
    ek.density()
    ek.force()
    fk = ek.download()["acc"]
    magk = np.linalg.norm(fk, axis=1)
    errk = np.linalg.norm(f32 - fk, axis=1) / np.maximum(magk, np.sqrt(np.mean(magk ** 2)))
    ek.set_tuning(1, skin)
    ek.step(2)
    ek.step(10)
    vk = n * 10 / (ek.last_step_ms() * 1e-3)
    ek.close()
    return {"workload": "mdpd_liquid_1m", "n_particles": int(n), "steps": steps,
            "equilibration_steps": equil, "tuning": tuned,
            "value": v32, "fp64_plain": v64, "speedup_fp32_over_fp64": v32 / v64,
            "fp64_same_algorithm": vk, "speedup_fp32_over_fp64_same_algorithm": v32 / vk,
            "force_error_vs_fp64_same_algorithm": float(errk.max()),
            "unit": "particle-steps/s",
            "force_error": {"max_rel": float(err.max()),
                            "aggregate": float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64))},
            "description": "55^3 periodic box at density 6, Warren form A -40, B 25, r_d 0.75, "
                           "sigma 3, dt 0.005, uniform random start"}


def replica_params(reps):
    """Warren-form parameters of the batched replicas (A per replica, B 25,
    r_d 0.75, sigma 3, dt 0.005, each replica's own seed)."""
    from implicit_dpd_gb300.abi import FORM_WARREN
    from implicit_dpd_gb300.engine import derive_params

    params = []
    for r in reps:
        p = derive_params(configs.run_param(r["box"], dt=0.005, cf_r=3.0))
        p.seed, p.time, p.form = r["seed"], 1, FORM_WARREN
        p.warren_a, p.warren_b, p.warren_rd = r["a"], 25.0, 0.75
        params.append(p)
    return params


def replica_observables_cpu(reps, rank, world, dist, steps=3):
    """The multi-rank replica path on the host: the replicas are dealt to the
    ranks by LPT on their particle counts, each rank steps its own (CPU
    oracle) and the per-replica kinetic temperatures are gathered in replica
    order. Returns the gathered temperatures, the owner rank of every replica
    and the replicas this rank stepped."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from implicit_dpd_gb300.partition import lpt_partition

    sizes = [len(r["state"]["pos"]) for r in reps]
    parts, _ = lpt_partition(sizes, world)
    params = replica_params(reps)
    mine = {}
    for i in parts[rank]:
        st = {k: np.array(v, copy=True) for k, v in reps[i]["state"].items()}
        p = params[i]
        for _ in range(steps):
            O.md_step(p, st)
        mine[i] = float((st["vel"] ** 2).sum() / (3.0 * len(st["vel"])))
    temps = {}
    for part in dist.gather(mine):
        temps.update({int(k): v for k, v in part.items()})
    owner = [next(k for k, p in enumerate(parts) if i in p) for i in range(len(reps))]
    return {"temperature": [temps[i] for i in range(len(reps))], "owner": owner,
            "stepped_here": sorted(parts[rank])}


def replicas_bench(steps=50, n_rep=256, device=0, rank=0, world=1, dist=None):
    """Batched MDPD replicas (256 liquids of 2k-60k particles, Warren form,
    A in [-50, -30], B = 25, densities 5-7): all of a rank's replicas in one
    handle, the steps of a call in one graph launch (and, for comparison, one
    graph launch per step), against the same replicas stepped one handle at
    a time with the same tuning (reach, skin and force-pass shape, picked by
    the package's tuner on the batch). On
    several ranks the replicas are dealt out by LPT on their particle counts
    (no exchange while stepping); the job's rate is all particles x steps
    over the slowest rank's time. Returns particle-steps/s of both forms."""
    from implicit_dpd_gb300.abi import CFG_PLAIN_GRAPHS
    from implicit_dpd_gb300.engine import Engine
    from implicit_dpd_gb300.partition import imbalance, lpt_partition

    dist = dist or Dist(1)
    reps = configs.mdpd_replicas(n_rep)
    sizes = [len(r["state"]["pos"]) for r in reps]
    parts, loads = lpt_partition(sizes, world)
    mine = parts[rank]
    params = replica_params(reps)
    n_tot = sum(sizes)
    eb = Engine(n_replicas=len(mine), device=device)
    for k, i in enumerate(mine):
        eb.set_params(params[i], k)
        eb.upload(reps[i]["state"], k)
    eb.step(3)
    # the package's tuner on the batch: (reach, skin), then the force pass's shape
    tuned, _ = autotune(eb, steps=20)
    reach, skin, lanes, blocks = tuned["reach"], tuned["skin"], tuned["lanes"], tuned["blocks"]
    dlanes = tuned["dens_lanes"]
    # every arm starts from this state (the batch after the tuner's ~270 steps)
    # and takes the same 3 warm-up steps, so all arms time the same trajectory
    start = [eb.download(replica=k) for k in range(len(mine))]
    t_start = [eb.get_params(k).time for k in range(len(mine))]

    def upload(e, k, replica):
        q = type(params[mine[k]]).from_buffer_copy(params[mine[k]])
        q.time = t_start[k]
        e.set_params(q, replica)
        s0 = start[k]
        e.upload({key: s0[key] for key in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")},
                 replica)

    for k in range(len(mine)):  # the same fresh start (lists built anew) as the other arms
        upload(eb, k, k)
    eb.step(3)
    dist.barrier()
    eb.step(steps)  # the steps in one graph launch (the step in a WHILE node)
    batched = n_tot * steps / (dist.max(eb.last_step_ms()) * 1e-3)
    # the same batch with one graph launch per step
    ep = Engine(n_replicas=len(mine), device=device, flags=CFG_PLAIN_GRAPHS)
    for k in range(len(mine)):
        upload(ep, k, k)
    ep.set_tuning(reach, skin, lanes=lanes, blocks=blocks, dens_lanes=dlanes)
    ep.step(3)
    dist.barrier()
    ep.step(steps)
    per_step_launch = n_tot * steps / (dist.max(ep.last_step_ms()) * 1e-3)
    ep.close()
    # what one persistent launch could save at most: the graph step's time
    # beyond its kernels' own times. Compared at skin 0, where every step does
    # the same work (cells and all passes): 20 graph steps against the mean of
    # 10 un-graphed profile steps (CUDA events between kernels; the events add
    # gaps of their own, so the difference is a lower bound on the gaps)
    eb.set_tuning(reach, 0.0)
    eb.step(3)
    eb.step(20)
    graph_ms = eb.last_step_ms() / 20
    prof = [eb.profile_step() for _ in range(10)]
    kernels_ms = sum(statistics.mean(p_[k] for p_ in prof) for k in prof[0])
    eb.close()
    singles = []
    for k in range(len(mine)):
        e = Engine(device=device)
        upload(e, k, 0)
        e.set_tuning(reach, skin, lanes=lanes, blocks=blocks, dens_lanes=dlanes)
        e.step(3)
        singles.append(e)
    import torch
    torch.cuda.synchronize()
    dist.barrier()
    t0 = time.perf_counter()
    for e in singles:  # one replica after the other, each its own graph launches
        e.step(steps)
    t1 = dist.max(time.perf_counter() - t0)
    one_at_a_time = n_tot * steps / t1
    for e in singles:
        e.close()
    return {"workload": "mdpd_replicas_256", "n_replicas": n_rep, "n_particles": int(n_tot),
            "steps": steps, "tuning": tuned,
            "batched": batched, "batched_per_step_launch": per_step_launch,
            "one_at_a_time": one_at_a_time,
            "launch": "batched: the steps of one idpd_step call in one graph launch (the "
                      "captured step repeated by a conditional WHILE node on the device); "
                      "batched_per_step_launch: one graph launch per step",
            "speedup": batched / one_at_a_time, "unit": "particle-steps/s",
            "launch_gaps": {"tuning": {"reach": reach, "skin": 0.0}, "graph_ms_per_step": graph_ms,
                            "kernels_ms_per_step": kernels_ms,
                            "share": max(0.0, graph_ms - kernels_ms) / graph_ms},
            "partition": {"ranks": world, "rule": "greedy LPT on particle counts",
                          "replicas_per_rank": [len(p) for p in parts],
                          "particles_per_rank": loads, "imbalance": imbalance(loads)},
            "description": "256 MDPD liquids (Warren form, A in [-50,-30], B 25, r_d 0.75, "
                           "densities 5-7, 2k-60k particles log-uniform) in one handle per rank "
                           "and one graph per step vs one handle per replica stepped in turn"}


def save_state(path, e, n_amp, box, layers, tune):
    out = e.download()
    np.savez(path, box=box, layers=layers, n_amp=n_amp, reach=tune["reach"], skin=tune["skin"],
             time=e.get_params().time,
             **{k: out[k] for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")})


def run_kernel_case(path, device=0, reach=0, skin=None):
    """Three graph-launched steps from a saved equilibrated state: few
    launches before the pair passes, for kernel profiles of one launch."""
    z = np.load(path)
    box, layers = z["box"], int(z["layers"])
    st = {k: z[k] for k in ("pos", "vel", "acc", "id", "prop", "amp_id", "unit")}
    rp = workload(box=box, layers=layers)[2]
    e = make_engine(st, int(z["n_amp"]), rp, device=device)
    reach = reach or int(z["reach"])
    skin = float(z["skin"]) if skin is None else skin
    e.set_tuning(reach, skin)
    e.step(3)
    e.sync()
    print(json.dumps({"kernel_case": workload_name(box, layers), "n_particles": len(st["pos"]),
                      "steps": 3, "reach": reach, "skin": skin}), flush=True)
    e.close()


# IDPD_CFG_PLAIN_GRAPHS with --plain-graphs: one graph launch per step and no
# conditional nodes, the form whose kernels ncu can trace (the same results)
GRAPH_FLAGS = 0


def make_engine(st, n_amp, rp, flags=0, device=0):
    from implicit_dpd_gb300.engine import Engine, derive_params

    p = derive_params(rp)
    p.seed, p.time = 12345, 1
    e = Engine(flags=flags | GRAPH_FLAGS, sort_period=100, device=device)
    e.set_params(p)
    e.upload(st)
    e.build_topology(n_amp)
    return e


def pinned(shape):
    import torch

    t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    return t, t.numpy()


def autotune(e, steps=40):
    """Times each (cell reach, skin), then each force-pass shape (lanes per
    particle, row blocks per CTA), on the current state over enough steps to
    include list rebuilds, and keeps the fastest (the package's tuner, without
    its cache: the bench measures afresh)."""
    from implicit_dpd_gb300.autotune import tune

    return tune(e, steps=steps)


def pair_roofline(kernel_ms, pairs, n, clocks, device, which=None):
    """Roofline of the dominant pair pass against its own bound, CUDA-core
    instruction issue: the algorithmic lane operations of the reference's
    pair work (OPS_PER_ORDERED_PAIR x the ordered pairs within the cutoff,
    counted on the device) over the kernel's CUDA-event time, against 4
    warp-instruction issue slots x 32 lanes x SMs x the sampled SM clock.
    The HBM figures and the ncu DRAM traffic of the same kernel ride along."""
    import torch

    top = which or max(PAIR_KERNELS, key=lambda k: kernel_ms[k])
    kinfo = PAIR_KERNELS[top]
    top_ms = kernel_ms[top]
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    ops = OPS_PER_ORDERED_PAIR[top] * pairs
    achieved = ops / (top_ms * 1e-3) / 1e12
    peak = 4.0 * 32.0 * sms * mhz * 1e6 / 1e12
    hbm_peak, peak_kind = measured_peaks()
    hbm = kinfo["bytes_per_particle"] * n / (top_ms * 1e-3) / 1e9
    traffic = profiled_traffic(kinfo["profile"])
    return {"kernel": kinfo["kernel"], "bound": "issue", "achieved": achieved, "peak": peak,
            "unit": "TOP/s", "frac": achieved / peak, "traffic": traffic,
            "kernel_ms": top_ms, "ordered_pairs": pairs, "pairs_per_bead": pairs / n,
            "ops_per_ordered_pair": OPS_PER_ORDERED_PAIR[top],
            "definition": "achieved = ops_per_ordered_pair x ordered pairs within the cutoff "
                          "(idpd_pair_count of the timed state) / the kernel's CUDA-event time; "
                          "peak = 4 issue slots x 32 lanes x SMs x median sampled SM clock "
                          f"({sms} SMs, {mhz:g} MHz); lane operations in 1e12/s",
            "evaluated_pairs_frac": achieved / peak / 2.0,
            "evaluated_pairs_note": "the engine evaluates each pair once (the reference twice): "
                                    "against its own evaluations the fraction is half",
            "hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s", "frac": hbm / hbm_peak,
                    "bytes_per_particle": kinfo["bytes_per_particle"],
                    "peak_source": f"{peak_kind} copy bandwidth (of {peak_kind})",
                    "traffic_over_algorithmic": (traffic / (kinfo["bytes_per_particle"] * n)
                                                 if traffic else None)}}


def gpu_launches(steps, kept, rebuilds, t0, n_reorders):
    """The kernels the timed steps launch: per step those of the captured
    step, the IF bodies that ran (rebuilds with kept lists, the drift removal
    at step counters that are multiples of 100), one count kernel per launch
    of the loop (split at each storage reorder) and the reorders' kernels."""
    cm = sum(1 for t in range(t0, t0 + steps) if t % 100 == 0)
    per = KERNELS_PER_KEPT_STEP if kept else KERNELS_PER_STEP
    return (steps * per + (rebuilds * KERNELS_PER_REBUILD if kept else 0) + cm * KERNELS_PER_CM
            + (n_reorders + 1) + n_reorders * KERNELS_PER_REORDER)


def step_roofline(roofline, n, ms_per_step):
    """The step against the sum of its passes' lower-bound times: the two pair
    passes at the issue bound (their algorithmic lane operations per ordered
    pair x the counted pairs over the peak issue rate), the rest of the step
    at the measured copy bandwidth (176 compulsory HBM bytes per
    particle-step)."""
    pairs, peak = roofline["ordered_pairs"], roofline["peak"] * 1e12
    hbm_peak, _ = measured_peaks()
    parts = {"force_ms": OPS_PER_ORDERED_PAIR["force"] * pairs / peak * 1e3,
             "density_ms": OPS_PER_ORDERED_PAIR["density"] * pairs / peak * 1e3,
             "hbm_ms": STEP_BYTES_PER_PARTICLE * n / (hbm_peak * 1e9) * 1e3}
    lower = sum(parts.values())
    return {"lower_bound_ms": lower, "ms_per_step": ms_per_step, "frac": lower / ms_per_step,
            "parts": parts,
            "definition": "sum of the passes' lower-bound times (pair passes at 4 issue slots x "
                          "32 lanes x SMs x clock for their algorithmic lane operations, the "
                          "rest at the measured copy bandwidth for 176 B per particle-step) "
                          "over the measured step"}


def fp64_arms(st64, n_amp, rp, tune, value32, steps, device):
    """Both FP64 arms on one state: particle-steps/s, the FP32 engine's
    speed-up over each, and the FP32 engine's pair-force error against each
    (pair passes only, same positions)."""
    from implicit_dpd_gb300.abi import CFG_FP64_KEPT, CFG_FP64_PAIRS

    e32 = make_engine(st64, n_amp, rp, device=device)
    e32.density()
    e32.force()
    f32 = e32.download()["acc"]
    e32.close()

    def arm(flags, kept):
        e = make_engine(st64, n_amp, rp, flags=flags, device=device)
        e.density()
        e.force()
        f64 = e.download()["acc"]
        mag = np.linalg.norm(f64, axis=1)
        floor = np.sqrt(np.mean(mag ** 2))
        err = np.linalg.norm(f32 - f64, axis=1) / np.maximum(mag, floor)
        if kept:
            e.set_tuning(1, tune["skin"])
        e.step(2)
        k = max(2, min(steps, 10))
        e.step(k)
        ms = e.last_step_ms()
        e.close()
        v = len(st64["pos"]) * k / (ms * 1e-3)
        return {"value": v, "unit": "particle-steps/s", "steps": k, "ms_per_step": ms / k,
                "speedup_fp32_over_fp64": value32 / v,
                "force_error": {"max_rel": float(err.max()),
                                "aggregate": float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64)),
                                "bar": 1e-5,
                                "definition": "per particle |F32 - F64| / max(|F64|, rms |F64|), "
                                              "pair forces of the timed state"}}

    plain = arm(CFG_FP64_PAIRS, False)
    plain["algorithm"] = "one thread per particle, 27 cells every step, each pair from both sides"
    same = arm(CFG_FP64_KEPT, True)
    same["algorithm"] = (f"the engine's: kept lists (reach 1, skin {tune['skin']:g}), each pair "
                         "once by its owner, fixed-point sums; FP64 pair arithmetic")
    return plain, same


def run_engine(args, rank, world, local_rank):
    dist = Dist(world)
    box, layers = np.asarray(args.box, np.float64), args.layers
    st, n_amp, rp = workload(box=box, layers=layers)
    n = len(st["pos"])
    e = make_engine(st, n_amp, rp, device=local_rank)
    # the lattice start compacts to the model's membrane density (~150
    # in-range neighbours per bead) within ~2000 steps: measure that state
    t_eq = time.perf_counter()
    e.step(args.equil)
    t_eq = time.perf_counter() - t_eq
    if args.reach:
        e.set_tuning(args.reach, args.skin, lanes=args.lanes, blocks=args.blocks)
        reach, tune_ms = e.tuning(), None
    else:
        reach, tune_ms = autotune(e)
    if args.save_state and rank == 0:
        save_state(args.save_state, e, n_amp, box, layers, reach)
    e.step(max(args.warmup, 3))
    dist.barrier()
    e.sync()
    rb0 = e.list_rebuilds()
    t0_step = e.get_params().time  # the step counter at the first timed step
    clk = Clocks(local_rank)
    clk.start()
    e.step(args.steps)  # CUDA events around the steps on the engine's stream
    ms = e.last_step_ms()
    clocks = clk.stop()
    rebuilds = e.list_rebuilds() - rb0
    dist.barrier()
    ms_max = dist.max(ms)
    value = n * args.steps * world / (ms_max * 1e-3)

    # per-kernel CUDA-event times of un-graphed steps (dominant kernel = force)
    pairs = e.pair_count()  # ordered pairs within the cutoff of the last timed step
    prof = [e.profile_step() for _ in range(5)]
    kernel_ms = {k: statistics.median(p_[k] for p_ in prof) for k in prof[0]}
    roofline = pair_roofline(kernel_ms, pairs, n, clocks, local_rank)
    # the other pair pass against the same issue bound, for reference
    other = [k for k in PAIR_KERNELS if PAIR_KERNELS[k]["kernel"] != roofline["kernel"]]
    if other:
        sec = pair_roofline(kernel_ms, pairs, n, clocks, local_rank, which=other[0])
        roofline["second_pass"] = {k: sec[k] for k in ("kernel", "achieved", "peak", "frac",
                                                         "kernel_ms", "ops_per_ordered_pair",
                                                         "traffic")}
    step_gbs = STEP_BYTES_PER_PARTICLE * n / (ms_max / args.steps * 1e-3) / 1e9

    # the FP64 arms of the metric on the timed state: the plain FP64 kernels
    # (one thread per particle, 27 cells, each pair from both sides) and the
    # engine's own algorithm in FP64 (kept lists, each pair once)
    fp64, fp64_same = None, None
    if not args.no_fp64:
        eq = e.download()
        st64 = dict(st, pos=eq["pos"], vel=eq["vel"], acc=eq["acc"])
        fp64, fp64_same = fp64_arms(st64, n_amp, rp, reach, value / world, args.steps,
                                    local_rank)

    # end to end through the C ABI: host pinned pos/vel/acc in, one step, out
    e2e = None
    if not args.no_e2e:
        tp, pos = pinned((n, 3))
        tv, vel = pinned((n, 3))
        ta, acc = pinned((n, 3))
        e.download_dynamics(pos, vel, acc)
        k2 = max(3, min(args.steps, 50))
        e.sync()
        t0 = time.perf_counter()
        for _ in range(k2):
            e.step_host(pos, vel, acc)
        t2 = time.perf_counter() - t0
        e.sync()
        t0 = time.perf_counter()
        for _ in range(k2):
            e.set_dynamics(pos, vel, acc)
            e.step(1)
            e.download_dynamics(pos, vel, acc)
        t3 = time.perf_counter() - t0
        e2e = {"value": n * k2 * world / dist.max(t2), "unit": "particle-steps/s",
               "h2d_bytes_per_step": 72 * n, "d2h_bytes_per_step": 72 * n, "steps": k2,
               "path": "idpd_step_host per step: pinned host pos/vel/acc in, one step, the new "
                       "pos/vel/acc out (positions copied back during the pair passes)",
               "three_calls": {"value": n * k2 * world / dist.max(t3),
                               "path": "idpd_set_dynamics + idpd_step(1) + idpd_download_state "
                                       "per step"}}

    batched = (replicas_bench(device=local_rank, rank=rank, world=world, dist=dist)
               if not args.no_replicas else None)
    reaction = reaction_bench(reach, device=local_rank) if not args.no_reaction else None
    liquid = liquid_bench(device=local_rank) if not args.no_liquid else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        timed_state = e.download()
        cpu = cpu_baseline(timed_state, n_amp, rp, e.get_params().time)
    n_reorders = args.steps // 100
    out = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "config": dict(workload_desc(n, n_amp, box, layers), equilibration_steps=args.equil,
                                               equilibration_s=t_eq, tuning=reach,
                                               autotune_ms_per_step=tune_ms,
                                               list_rebuilds_in_timed_steps=rebuilds,
                                               pairs_per_bead=pairs / n,
                                               parallelism=f"replicas{world}" if world > 1 else "single"),
           "clocks": clocks, "roofline": roofline, "step_hbm_gbs": step_gbs,
           "step_roofline": step_roofline(roofline, n, ms_max / args.steps),
           "kernel_ms": kernel_ms, "fp64_plain": fp64, "fp64_same_algorithm": fp64_same,
           "e2e": e2e, "cpu_baseline": cpu,
           "batched_replicas": batched, "reaction": reaction, "liquid": liquid,
           # per step its kernels and the loop's tail node; per launch of the
           # loop its count kernel (one launch, split at each reorder)
           "gpu_launches": gpu_launches(args.steps, reach["skin"] > 0, rebuilds, t0_step,
                                        n_reorders),
           "force_error_bar": "max-particle relative force error <= 1e-5 vs FP64 (tests/test_gpu_parity.py)"}
    if rank == 0:
        print(json.dumps(out), flush=True)
    e.close()
    dist.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--equil", type=int, default=2000,
                    help="untimed steps that take the lattice start to the membrane's density")
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-replicas", action="store_true")
    ap.add_argument("--no-reaction", action="store_true",
                    help="skip the membrane-with-precursor line")
    ap.add_argument("--no-liquid", action="store_true",
                    help="skip the 10^6-particle MDPD liquid line")
    ap.add_argument("--box", type=float, nargs=3, default=list(BOX),
                    help="periodic box of the stacked-bilayer workload")
    ap.add_argument("--layers", type=int, default=N_LAYERS, help="bilayers stacked along z")
    ap.add_argument("--save-state", default=None,
                    help="write the equilibrated state (npz) for --kernel-case")
    ap.add_argument("--plain-graphs", action="store_true",
                    help="one graph launch per step and no conditional nodes (for ncu)")
    ap.add_argument("--kernel-case", default=None,
                    help="load a saved state and run three graph steps (profiling case)")
    ap.add_argument("--liquid-case", type=int, default=None, metavar="STEPS",
                    help="the MDPD liquid at its tuned shape: STEPS graph steps, then 12 "
                         "(profiling case)")
    ap.add_argument("--reach", type=int, default=0,
                    help="cell reach (1 or 2) instead of the autotuned one")
    ap.add_argument("--skin", type=float, default=0.0,
                    help="neighbour-list skin with --reach (0: lists every step)")
    ap.add_argument("--lanes", type=int, default=16,
                    help="force pass: lanes per particle with --reach (8, 16 or 32)")
    ap.add_argument("--blocks", type=int, default=1,
                    help="force pass: 128-row blocks per CTA with --reach (1, 2 or 4)")
    args = ap.parse_args()
    if args.plain_graphs:
        from implicit_dpd_gb300.abi import CFG_PLAIN_GRAPHS

        global GRAPH_FLAGS
        GRAPH_FLAGS = CFG_PLAIN_GRAPHS
    rank, world, local_rank = dist_env()
    if args.kernel_case:
        run_kernel_case(args.kernel_case, local_rank, args.reach,
                        args.skin if args.reach else None)
        return
    if args.liquid_case is not None:
        run_liquid_case(args.liquid_case, local_rank)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    run_engine(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
