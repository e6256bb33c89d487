"""Benchmark of the GB300 DEM step engine.

One "step" is one pass of the reference's step loop (advance, force
evaluation, finish, host MBD) over the whole scene.  Default workload: the
rotating drum of 2,000,000 lognormal spheres (median 1 mm, sigma 0.25,
clipped to [0.5, 2] mm) in a 19,520-triangle cylinder of radius 0.3 m and
length 0.5 m turning at 2 rad/s, dt = 2e-6 s, seeded synthetic bed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--config c2|c1|c0|c4] [--precision mixed|fp64]

Prints one JSON line.  ``value`` is particle-steps/s of the headline
precision with the state resident in HBM (CUDA events on the engine stream);
``e2e`` is the same metric through the C ABI per step (body states uploaded
and body loads read back every step, as the reference's host loop does);
``reference_fp64_cuda`` times the reference's own FP64 CUDA kernels on the
same GPU and scenes.  With --gpus N > 1 outside torchrun, the script starts
N ranks itself.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
# pipeline phases timed with CUDA events in one force evaluation
PHASES = ["grid", "triangles+gather", "sweep", "walls", "pp_law", "pt_items", "pt_law", "owner_sum", "body_reduce"]


def make_scene(config, particles=None):
    from dem_mbd_cuda_gb300 import generate as G
    if config == "c0":
        n = particles or 20000
        return G.pure_dem(n=n, seed=1000), "pure DEM, %d spheres r~U[1.8,2.2] mm on a lattice, 5 walls, dt 1e-5" % n
    if config == "c4":
        scenes = G.batch(settled=True)
        n = sum(sc.n for sc in scenes)
        return scenes, ("256 independent box scenes (0.1 x 0.1 x 0.4 m, 5 walls), N_s ~ U[2000, 40000], "
                        "%d spheres in total, per-scene friction and restitution, settled in columns, one engine" % n)
    if config == "c2":
        n = particles or 2000000
        sc, _ = G.drum(n=n, seed=1002)
        return sc, ("rotating drum (R 0.3 m, L 0.5 m, 2 rad/s), %d lognormal spheres (median 1 mm, sigma 0.25, "
                    "clipped to [0.5, 2] mm) settled in hexagonal columns and co-rotating, filling 45%% of the drum "
                    "(config: 40%%, a solid fraction of 0.2 for 2M spheres), %d-triangle cylinder, friction 0.5, "
                    "restitution 0.3, kN 1e5, dt 2e-6" % (n, sc.n_triangles))
    n = particles or 200000
    sc, _ = G.mbd_blade_plate(n=n, seed=1001)
    return sc, ("DEM-MBD, %d spheres r~U[1.5,2.5] mm settled in columns in a 0.4 m box, %d-triangle blade "
                "(omega_z 3) + %d-triangle 1 kg plate, dt 5e-6"
                % (n, int((sc.tri_body == 0).sum()), int((sc.tri_body == 1).sum())))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=None):
        # nvidia-smi counts physical GPUs: the process's GPU is the first
        # visible one (an index or a UUID, both accepted by -i)
        if index is None:
            index = (os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip() or "0")
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"]
        try:
            self._proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._thread = threading.Thread(target=self._read, daemon=True)
            self._thread.start()
        except Exception:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def algorithmic_bytes(n, nc, contacts, wall_contacts, body_manifolds, triangles, h):
    """Per-step algorithmic bytes of the whole pipeline:
    N*412 + Nc*24 + (C_pp + C_pw + C_pb)*2*(8 + 9h) + T*288, with C_pp the
    unordered particle contacts (= contact sides / 2)."""
    return n * 412 + nc * 24 + (contacts / 2 + wall_contacts + body_manifolds) * 2 * (8 + 9 * h) + triangles * 288


# Algorithmic DRAM bytes of one launch of the single-kernel phases, from the
# data each must move once (records, cell rows, history, contact list), for
# n particles with s contact sides; hv = bytes of one history slot.
KERNEL_BYTES = {
    # own record (relf, pos, meta, cell) 80 + counters 12 + three high-water
    # marks 12 + history key and age 12/slot; contact list entry 16 + key and
    # age 12 per side; the cells: 9 cell-row boundaries 144, or (neighbour
    # lists, mean length L) the list count 4 and per entry its index and the
    # partner's sorted position 8
    "sweep": ("k_sweep", lambda n, s, hv, L=None: n * (116 + (144 if L is None else 4 + 8 * L)) + s * 28),
    # per side: list entry 16, history slot read + write, result row 24;
    # per particle: its FP64 position 32 and four FP32 rows 64
    "pp_law": ("k_pp_law", lambda n, s, hv: s * (16 + 2 * hv + 24) + n * 96),
    # per owner: count, flags, field force, inverse mass and inertia,
    # quaternion, omega, accelerations; result rows 24 per side
    "owner_sum": ("k_owner_sum", lambda n, s, hv: n * 196 + s * 24),
}


def pt_bytes(items, manifolds, hv_body):
    """Algorithmic bytes of the particle-triangle law kernel (k_pt_warp or
    k_pt_thread): per contact item its cell, record and owner state 208 B;
    per manifold the body history slot read and written and its load record
    (32 doubles).  Triangle rows are shared by the items of a cell and not
    counted."""
    return items * 208 + manifolds * (2 * hv_body + 32 * 8)


def dominant_kernel(phases, n, sides, hv, list_length=None, items=0, manifolds=0):
    """The single-kernel phase that takes longest (sweep, particle law,
    particle-triangle law or owner sum) and its roofline inputs."""
    times = dict(zip(PHASES, phases))
    cands = list(KERNEL_BYTES) + (["pt_law"] if items else [])
    name = max(cands, key=lambda k: times.get(k, 0.0))
    if name == "pt_law":
        kernel = "k_pt_thread" if items > 3072 else "k_pt_warp"
        return name, kernel, times[name], pt_bytes(items, manifolds, 108)
    kernel, fn = KERNEL_BYTES[name]
    nbytes = fn(n, sides, hv, list_length) if name == "sweep" else fn(n, sides, hv)
    return name, kernel, times[name], nbytes


def traffic_record(kernel, config):
    """The committed ncu capture of a kernel on a workload
    (profiles/traffic.json: read + write DRAM bytes per particle at a stated
    scene size, FP64 pipe activity), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)[config][kernel]
    except Exception:
        return None


def measured_traffic(kernel, n, config):
    """DRAM bytes of one launch from the kernel's capture, scaled to n
    particles (per-particle traffic measured on a smaller scene of the same
    generator); None when there is no capture."""
    rec = traffic_record(kernel, config)
    return (rec["bytes_per_particle"] * n, rec["source"]) if rec else (None, None)


def launches_per_step(scene):
    """Kernels one graph-launched step issues (the force DAG of
    dem_engine.cu enqueue_forces, steady-state step)."""
    # counters x2, grid keys + layout + count + scan + scatter + place,
    # geometry gather, sweep, particle law, owner sum, position advance;
    # rotational branch: rotational advance, velocity gather
    k = 2 + 6 + 1 + 1 + 1 + 1 + 1 + 2
    if scene.comp_owner is not None:
        k += 1                   # component update
    if scene.universal_gravity_enabled:
        k += 1
    if scene.n_walls:
        k += 2                   # wall probe + law
    if scene.n_bodies and scene.n_triangles:
        k += 5 + 3 + 2           # triangle transform + grid, PT items + the two law kernels, body reduction
    elif scene.n_bodies:
        k += 2
    return k


def run_engine(scene, precision, steps, warmup):
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    e = CudaDemSolver().initialize(scene, precision=precision)
    e.run(max(1, warmup))
    with ClockSampler() as clk:
        ms = e.time_steps(steps)
    stats = e.stepStats()
    # per-kernel times: CUDA events on the engine stream around each phase
    # of five force evaluations after the timed region, averaged
    nl = e.neighbor_stats()
    nl["steps"] = max(1, warmup) + steps
    runs = [e.compute_forces_timed(diag=(k == 4)) for k in range(5)]
    phases = [sum(r[k] for r in runs) / len(runs) for k in range(len(runs[0]))]
    stats_after = e.stepStats()
    stats_after["neighbor_lists"] = nl
    return e, ms, clk.summary(), stats, phases, stats_after


def e2e_run(scene, precision, steps, warmup):
    """Per-step calls through the C ABI: body states H2D from host memory and
    body loads D2H every step (dem_run_steps(1) per call)."""
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    e = CudaDemSolver().initialize(scene, precision=precision)
    e.run(max(1, warmup))
    t0 = time.perf_counter()
    for _ in range(steps):
        e.run(1)
    t1 = time.perf_counter()
    return (t1 - t0) * 1000.0


def cpu_baseline(scene, budget_s=12.0, threads=None):
    from oracle.oracle import Oracle
    threads = threads or os.cpu_count() or 1
    o = Oracle(scene, threads=threads)
    o.run(1)
    done = 0
    t0 = time.perf_counter()
    while True:
        o.run(1)
        done += 1
        if time.perf_counter() - t0 >= budget_s or done >= 200:
            break
    dt = time.perf_counter() - t0
    return scene.n * done / dt, threads, done, dt


def load_error(scene, evaluations=3):
    """Error of the mixed form against the FP64 form, body loads and particle
    forces, over the first evaluations of the reference's step sequence
    (evaluation 0 has dt = 0; later ones start from states that differ only by
    the previous step's force difference times dt^2).  Reported for the
    default mixed form (particle-triangle law in FP64) and with the
    particle-triangle law in FP32 as well."""
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    out = {}
    for label, kw in (("mixed", {}), ("mixed_pt_fp32", {"pt_fp32": True})):
        a = CudaDemSolver().initialize(scene, precision="fp64")
        b = CudaDemSolver().initialize(scene, precision="mixed", **kw)
        bs = scene.body_states() if scene.n_bodies else None
        dt = scene.dt
        load_err, force_err = [], []
        for k in range(evaluations):
            if k == 1:
                a.initializeParticleHalfStep(0.5 * dt)
                b.initializeParticleHalfStep(0.5 * dt)
            if k >= 1:
                a.advanceParticles(dt)
                b.advanceParticles(dt)
            la = a.computeForces(k * dt, bs, True, True)
            lb = b.computeForces(k * dt, bs, True, True)
            fa = a.downloadForceOutput(False, False)["total"]
            fb = b.downloadForceOutput(False, False)["total"]
            force_err.append(float(np.abs(fa - fb).max() / max(np.abs(fa).max(), 1e-30)))
            if la is not None and len(la):
                load_err.append(float(np.abs(la - lb).max() / max(np.abs(la).max(), 1e-30)))
            a.finishParticleStep(dt)
            b.finishParticleStep(dt)
        out[label] = {"force_rel_err_max": force_err, "body_load_rel_err": load_err}
        if scene.n_bodies == 0:
            break
    return out


def wall_contacts(e, scene):
    """Particle-wall contacts of the engine's last evaluation (wall history
    slots seen in the latest step)."""
    if not scene.n_walls:
        return 0
    keys, last, _ = e.history(1)
    used = keys != 0
    return int((used & (last == last[used].max())).sum()) if used.any() else 0


def roofline(phases, scene, stats, nlists, precision, e, per_step_ms, config):
    """Roofline of the dominant kernel (CUDA-event time of its phase) and the
    step-level algorithmic bytes (section (d) of the design notes)."""
    h = 4 if precision == "mixed" else 8
    hv = 3 * h * 4            # one history slot: 9 values padded to 12
    contacts = stats["particle_contacts"]
    peak, peak_kind = hbm_peak()
    pname, kernel, kms, kbytes = dominant_kernel(phases, scene.n, contacts, hv, nlists["mean_length"],
                                                 stats.get("body_candidate_items", 0), stats["body_contacts"])
    achieved = kbytes / (kms / 1000.0) / 1e9
    traffic, traffic_src = measured_traffic(kernel, scene.n, config)
    step_bytes = algorithmic_bytes(scene.n, scene.n_components, contacts, wall_contacts(e, scene),
                                   stats["body_contacts"], scene.n_triangles, h)
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "traffic": traffic, "kernel": kernel, "phase": pname, "kernel_ms": kms,
           "algorithmic_bytes": kbytes, "traffic_source": traffic_src, "peak_kind": peak_kind + " (hbm_gbs)",
           "step": {"algorithmic_bytes": step_bytes, "achieved": step_bytes / (per_step_ms / 1000.0) / 1e9}}
    if pname == "pt_law":
        # a chain of FP64 arithmetic per contact item: its HBM figure is
        # beside the point, the FP64 pipe's activity is in fp64_roofline
        out["note"] = "FP64-latency bound per contact item; see fp64_roofline for the FP64 pipe activity"
    return out


def fp64_roofline(phases, config, precision):
    """FP64-bound kernels (the FP64 form's particle law, the particle-triangle
    law): their phase time and the FP64 pipe's activity in their ncu
    capture (sm__pipe_fp64_cycles_active, % of peak)."""
    times = dict(zip(PHASES, phases))
    out = {}
    for phase, kernel in (("pp_law", "k_pp_law<double>" if precision == "fp64" else None), ("pt_law", "k_pt_thread"),
                          ("pt_law", "k_pt_warp")):
        rec = traffic_record(kernel, config) if kernel else None
        if rec and rec.get("fp64_pipe_pct") is not None:
            out[kernel] = {"phase_ms": times.get(phase), "fp64_pipe_active_frac": rec["fp64_pipe_pct"] / 100.0,
                           "source": rec["source"]}
    return out


def scene_summary(config, steps, warmup):
    """A workload in both precisions, its phases, the dominant kernel's
    roofline and the mixed form's error against FP64."""
    scene, desc = make_scene(config)
    out = {"workload": desc, "particles": scene.n, "triangles": scene.n_triangles}
    for prec in ("mixed", "fp64"):
        e, ms, clocks, stats, phases, after = run_engine(scene, prec, steps, warmup)
        out[prec] = {"value": scene.n * steps / (ms / 1000.0), "ms_per_step": ms / steps,
                     "contact_sides_per_step": stats["particle_contacts"],
                     "body_manifolds": stats["body_contacts"], "phase_ms": dict(zip(PHASES, phases)),
                     "neighbor_lists": after["neighbor_lists"], "clocks": clocks,
                     "roofline": roofline(phases, scene, stats, after["neighbor_lists"], prec, e, ms / steps, config),
                     "fp64_roofline": fp64_roofline(phases, config, prec)}
        del e
    out["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["load_error_vs_fp64"] = load_error(scene)
    return out


def host_cpu():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def reference_cuda_summary(configs, steps, warmup):
    """The reference's own FP64 CUDA path on this GPU: its kernels, built
    from its src/cuda/*.cu for sm_103a (oracle/_ref/ref_engine.cubin), driven
    by oracle/ref_cuda_host.cu, a restatement of its host loop with the same
    launches, Thrust calls, synchronous copies and host MBD step on one host
    thread.  Wall-clock time of `steps` steps after `warmup` steps, device
    synchronised on both sides."""
    from oracle import ref_cuda
    if not ref_cuda.available():
        return {"unavailable": "the reference's device code was not built (oracle/reference_build.py needs the "
                               "reference tree where the repository is built)"}
    ref_cuda.build()
    out = {"kind": "reference FP64 CUDA kernels (src/cuda/*.cu, sm_103a) with its host loop restated",
           "host": {"cpu": host_cpu(), "cores": os.cpu_count(), "host_threads_used": 1}}
    for config in configs:
        scene, desc = make_scene(config)
        r = ref_cuda.RefCuda(scene)
        r.run(max(1, warmup))
        k = max(1, min(steps, 20))
        sec = r.time_run(k)
        out[config] = {"workload": desc, "ms_per_step": 1e3 * sec / k, "value": scene.n * k / sec,
                       "unit": "particle-steps/s", "steps": k, "warmup": max(1, warmup)}
        del r
    return out


def batch_summary(steps, warmup):
    """The 256-scene batch (config 4) in both precisions: every scene advances
    in the same graph launch per step."""
    scenes, desc = make_scene("c4")
    n = sum(sc.n for sc in scenes)
    out = {"workload": desc, "scenes": len(scenes), "particles": n}
    for prec in ("mixed", "fp64"):
        e, ms, clocks, stats, phases, _ = run_engine(scenes, prec, steps, warmup)
        out[prec] = {"value": n * steps / (ms / 1000.0), "ms_per_step": ms / steps,
                     "contact_sides_per_step": stats["particle_contacts"], "phase_ms": dict(zip(PHASES, phases)),
                     "clocks": clocks}
        del e
    return out


def adjoint_summary(steps=2000, checkpoint_every=100):
    """Config 3: reverse-mode gradients of the mean particle height plus the
    sum of the dynamic plate's final centre coordinates with respect to the
    materials and the initial velocities.  Wall-clock times of a plain FP64
    forward run, the checkpointed forward run and the backward run
    (recompute + reverse sweep)."""
    from dem_mbd_cuda_gb300 import generate as G
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    scene = G.adjoint_settle()
    n = scene.n
    plain = CudaDemSolver().initialize(scene, precision="fp64")
    plain.run(0)
    plain.synchronize()
    t0 = time.perf_counter()
    plain.run(steps)
    plain.synchronize()
    t_plain = time.perf_counter() - t0
    del plain
    e = CudaDemSolver().initialize(scene, precision="fp64")
    t0 = time.perf_counter()
    e.adjoint_forward(steps, checkpoint_every)
    t_fwd = time.perf_counter() - t0
    dpos = np.zeros((n, 3))
    dpos[:, 2] = 1.0 / n
    dplate = np.ones((scene.n_bodies, 3))
    t0 = time.perf_counter()
    g = e.adjoint_backward(dpos, None, dl_dbody_center=dplate)
    t_bwd = time.perf_counter() - t0
    mem = e.adjoint_memory()
    plate_final = e.bodies()["center"][0].tolist()
    # finite-difference check at short horizons (FP64 central differences,
    # relative step 1e-6) on the same generator at 2,000 spheres: with many
    # colliding pairs a perturbed run crosses contact-onset steps (jumps of
    # the piecewise-smooth loss), which the frozen-contact-set derivative does
    # not contain; a smaller bed keeps the differences in the smooth range
    fd = {}
    import dataclasses

    def fd_rows(scene, hor, dpos, dplate, keys, rel=1e-6):
        ea = CudaDemSolver().initialize(scene, precision="fp64").adjoint_forward(hor, min(checkpoint_every, hor))
        ga = ea.adjoint_backward(dpos, None, dl_dbody_center=dplate)
        del ea

        def final(sc):
            ef = CudaDemSolver().initialize(sc, precision="fp64")
            ef.run(hor)
            return ef.downloadParticleState()["pos"][:, 2], ef.bodies()["center"]

        row = {}
        for cls, key in keys:
            m = getattr(scene, cls)
            x0 = getattr(m, key)
            h = rel * abs(x0)
            zp, cp = final(dataclasses.replace(scene, **{cls: dataclasses.replace(m, **{key: x0 + h})}))
            zm, cm = final(dataclasses.replace(scene, **{cls: dataclasses.replace(m, **{key: x0 - h})}))
            # differences taken per particle before the sums (exact for close
            # values), so the loss's own magnitude adds no rounding
            f = (float(np.mean(zp - zm)) + float(np.sum(cp - cm))) / (2 * h)
            a = ga["dl_dparams"][cls][key]
            row[f"{cls}.{key}"] = {"adjoint": a, "fd": f, "rel_err": abs(a - f) / max(abs(f), 1e-300)}
        return row

    # the bed without its plate at 50 and 200 steps: the plate lands on the
    # highest spheres, where the onset and break of its contacts make the
    # loss jump under a perturbation
    scene = G.adjoint_settle(n=2000, plate=False)
    dpos = np.zeros((scene.n, 3))
    dpos[:, 2] = 1.0 / scene.n
    for hor in (50, 200):
        fd[f"{hor}_steps"] = fd_rows(scene, hor, dpos, None, (("pp", "mu"), ("pp", "kN"), ("pp", "epsN"),
                                                              ("pw", "mu"), ("pw", "epsN")))
    # the plate term with the plate in contact from the first step: a 10 g
    # plate resting on 16 spheres (the particle-triangle material without
    # caps, so that no contact sits on a cap); its gradients are small, so a
    # relative step of 1e-5 keeps the differences above FP64's resolution
    mono = G.plate_on_monolayer()
    dmono = np.zeros((mono.n, 3))
    dmono[:, 2] = 1.0 / mono.n
    fd["plate_on_monolayer_60_steps"] = fd_rows(mono, 60, dmono, np.ones((1, 3)),
                                                (("pt", "kN"), ("pt", "epsN"), ("pt", "epsS"), ("pw", "kN")), rel=1e-5)
    return {"workload": "%d spheres r~U[1.8,2.2] mm settling in a 0.1 m box of 5 walls, v0 ~ N(0, 0.05 m/s), the "
                        "config-1 plate (1 kg, dynamic) resting on the bed, %d steps of dt 1e-5, checkpoints every "
                        "%d; loss = mean particle height + sum of the plate's final centre coordinates"
                        % (n, steps, checkpoint_every),
            "forward_plain_s": t_plain, "forward_checkpointed_s": t_fwd, "backward_s": t_bwd,
            "adjoint_over_forward": t_bwd / t_plain, "total_over_forward": (t_fwd + t_bwd) / t_plain,
            "memory": mem, "plate_final_center": plate_final,
            "dl_dparams": g["dl_dparams"], "dl_dvel0_norm": float(np.linalg.norm(g["dl_dvel0"])),
            "fd_check": fd}


def _scene_heights(pos, counts):
    """Mean particle height of each scene of a batch (the bed height's
    measure used as the calibration's loss)."""
    out, off = [], 0
    for c in counts:
        out.append(pos[off:off + c, 2].mean())
        off += c
    return out


def batch_adjoint_summary(nscenes=64, steps=50, checkpoint_every=10):
    """Config 4's batched reverse mode on the first `nscenes` settled scenes
    of the 256-scene generator (contact-dense beds, the reverse mode's most
    expensive regime): the gradients of the sum of the scenes' mean bed
    heights with respect to every scene's own materials and initial
    velocities, from one backward run over the batch, with the reverse law
    of the particle and wall contacts in FP64 and in FP32 (the forward run,
    its recompute and the rest of the reverse stay FP64), and the FP32 form's
    departure from the FP64 gradients."""
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    scenes = make_scene("c4")[0][:nscenes]
    n = sum(sc.n for sc in scenes)
    plain = CudaDemSolver().initialize(scenes, precision="fp64")
    plain.run(0)
    plain.synchronize()
    t0 = time.perf_counter()
    plain.run(steps)
    plain.synchronize()
    t_plain = time.perf_counter() - t0
    del plain
    dpos = np.zeros((n, 3))
    off = 0
    for sc in scenes:
        dpos[off:off + sc.n, 2] = 1.0 / sc.n
        off += sc.n
    out = {"workload": "the first %d settled scenes of the 256-scene batch (%d spheres), %d steps of dt 1e-5, "
                       "checkpoints every %d; loss = sum over scenes of the mean bed height"
                       % (nscenes, n, steps, checkpoint_every), "forward_plain_s": t_plain}
    grads = {}
    for form in ("fp64", "fp32"):
        e = CudaDemSolver().initialize(scenes, precision="fp64").set_adjoint_fp32(form == "fp32")
        t0 = time.perf_counter()
        e.adjoint_forward(steps, checkpoint_every)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        g = e.adjoint_backward(dpos, None)
        t_bwd = time.perf_counter() - t0
        out["reverse_" + form] = {"forward_checkpointed_s": t_fwd, "backward_s": t_bwd,
                                  "adjoint_over_forward": t_bwd / t_plain,
                                  "total_over_forward": (t_fwd + t_bwd) / t_plain, "memory": e.adjoint_memory()}
        grads[form] = g
        del e
    a, b = grads["fp64"], grads["fp32"]
    rel = [abs(b["dl_dparams"][k][c][f] - a["dl_dparams"][k][c][f]) / abs(a["dl_dparams"][k][c][f])
           for k in range(nscenes) for c in ("pp", "pw") for f in ("kN", "epsN", "epsS")
           if abs(a["dl_dparams"][k][c][f]) > 1e-12]
    out["fp32_vs_fp64"] = {"material_rel_err_median": float(np.median(rel)) if rel else 0.0,
                           "material_rel_err_p99": float(np.percentile(rel, 99)) if rel else 0.0,
                           "dl_dvel0_rel_err": float(np.abs(b["dl_dvel0"] - a["dl_dvel0"]).max()
                                                     / max(np.abs(a["dl_dvel0"]).max(), 1e-300))}
    out["per_scene_pp_depsN"] = [p["pp"]["epsN"] for p in a["dl_dparams"][:4]]
    return out


def calibration_summary(nscenes=16, steps=1000, iterations=4, checkpoint_every=100):
    """Config 4's calibration on its own scenes (jittered lattices that fall
    and settle): each scene's restitution is recovered from its bed height
    by Newton steps on the batched reverse mode's gradients
    (autograd.simulate_batch, one backward run for all scenes per
    iteration).  The horizon is the one where the reverse mode's gradients
    of this loss match central differences (measured: 1,000 steps); later,
    the bed's collisions make the height a non-smooth function of the
    restitution."""
    import dataclasses

    import torch
    from dem_mbd_cuda_gb300 import generate as G
    from dem_mbd_cuda_gb300.autograd import materials, simulate_batch
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    scenes = G.batch(nscenes=nscenes)
    counts = [s.n for s in scenes]
    true_e = np.array([s.pp.epsN for s in scenes])
    ref = CudaDemSolver().initialize(scenes, precision="fp64")
    ref.run(steps)
    target = np.array(_scene_heights(ref.downloadParticleState()["pos"], counts))
    del ref
    e = np.clip(true_e + np.where(np.arange(nscenes) % 2 == 0, 0.15, -0.15), 0.1, 0.9)
    vel0 = torch.tensor(np.concatenate([s.vel for s in scenes]))
    log = []
    t0 = time.perf_counter()
    for it in range(iterations + 1):
        pp = torch.stack([materials(dataclasses.replace(s.pp, epsN=float(x))) for s, x in zip(scenes, e)])
        pw = torch.stack([materials(dataclasses.replace(s.pw, epsN=float(x))) for s, x in zip(scenes, e)])
        pp.requires_grad_(True)
        pw.requires_grad_(True)
        pos, _ = simulate_batch(scenes, steps, pp, pw, vel0, checkpoint_every)
        h = torch.stack(_scene_heights(pos, counts))
        resid = h.detach().numpy() - target
        log.append({"iteration": it, "height_residual_max_m": float(np.abs(resid).max()),
                    "restitution_error_max": float(np.abs(e - true_e).max())})
        if it == iterations:
            break
        h.sum().backward()
        dh = (pp.grad[:, 2] + pw.grad[:, 2]).numpy()
        step = np.where(np.abs(dh) > 1e-30, resid / np.where(np.abs(dh) > 1e-30, dh, 1.0), 0.0)
        e = np.clip(e - step, 0.05, 0.95)
    return {"workload": "%d config-4 scenes (%d spheres, jittered lattices settling in 0.1 m boxes), %d steps of "
                        "dt 1e-5; unknown: each scene's restitution (particle and wall), from its mean bed height"
                        % (nscenes, sum(counts), steps),
            "iterations": log, "seconds": time.perf_counter() - t0}


def c4_adjoint_summary(chunk_particles=1_400_000, steps=3000, checkpoint_every=100):
    """The whole of config 4 in reverse mode: 256 scenes (5.46M spheres,
    jittered lattices settling) over 3,000 steps, the gradients of every
    scene's mean bed height with respect to its materials and initial
    velocities.  Scenes are independent, so the batch runs in chunks of up
    to `chunk_particles` spheres, one after the other on the GPU (the
    checkpoints and two segment tapes of the whole batch would not fit
    beside each other); times are summed over the chunks.  FP32 reverse law
    for the particle and wall contacts."""
    from dem_mbd_cuda_gb300 import generate as G
    from dem_mbd_cuda_gb300.engine import CudaDemSolver
    scenes = G.batch()
    chunks, cur, size = [], [], 0
    for s in scenes:
        if cur and size + s.n > chunk_particles:
            chunks.append(cur)
            cur, size = [], 0
        cur.append(s)
        size += s.n
    chunks.append(cur)
    t_plain = t_fwd = t_bwd = 0.0
    peak = {"checkpoint_bytes": 0, "tape_bytes": 0}
    nonzero = 0
    for ch in chunks:
        n = sum(s.n for s in ch)
        p = CudaDemSolver().initialize(ch, precision="fp64")
        p.run(0)
        p.synchronize()
        t0 = time.perf_counter()
        p.run(steps)
        p.synchronize()
        t_plain += time.perf_counter() - t0
        del p
        e = CudaDemSolver().initialize(ch, precision="fp64").set_adjoint_fp32(True)
        t0 = time.perf_counter()
        e.adjoint_forward(steps, checkpoint_every)
        t_fwd += time.perf_counter() - t0
        dpos = np.zeros((n, 3))
        off = 0
        for s in ch:
            dpos[off:off + s.n, 2] = 1.0 / s.n
            off += s.n
        t0 = time.perf_counter()
        g = e.adjoint_backward(dpos, None)
        t_bwd += time.perf_counter() - t0
        mem = e.adjoint_memory()
        peak = {k: max(peak[k], mem[k]) for k in peak}
        per = g["dl_dparams"] if isinstance(g["dl_dparams"], list) else [g["dl_dparams"]]
        nonzero += sum(1 for r in per if r["pp"]["epsN"] != 0.0 or r["pw"]["epsN"] != 0.0)
        del e
    return {"workload": "all 256 config-4 scenes (%d spheres, jittered lattices settling), %d steps of dt 1e-5, "
                        "checkpoints every %d, in %d chunks of up to %d spheres"
                        % (sum(s.n for s in scenes), steps, checkpoint_every, len(chunks), chunk_particles),
            "forward_plain_s": t_plain, "forward_checkpointed_s": t_fwd, "backward_s": t_bwd,
            "adjoint_over_forward": t_bwd / t_plain, "total_over_forward": (t_fwd + t_bwd) / t_plain,
            "peak_chunk_memory": peak, "scenes_with_restitution_gradient": nonzero}


def autotune_summary(scene, precision):
    """The autotuner's choice of cell factor, sweep blocks per SM and
    particle-triangle crossover on the workload (dem_mbd_cuda_gb300/autotune.py)."""
    from dem_mbd_cuda_gb300.autotune import autotune
    return autotune(scene, precision=precision)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c2", choices=["c0", "c1", "c2", "c4"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-drum", action="store_true", help="skip the embedded 2M-sphere drum summary")
    ap.add_argument("--no-c1", action="store_true", help="skip the embedded config-1 (200k DEM-MBD) summary")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip the timing of the reference's FP64 CUDA kernels")
    ap.add_argument("--no-batch", action="store_true", help="skip the embedded 256-scene batch summary")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the embedded config-3 adjoint summary")
    ap.add_argument("--no-autotune", action="store_true", help="skip the embedded autotuner summary")
    ap.add_argument("--adjoint-only", action="store_true", help="print the config-3 adjoint summary alone")
    ap.add_argument("--adjoint-c4", action="store_true",
                    help="print the reverse mode over all 256 config-4 scenes and 3,000 steps alone")
    ap.add_argument("--adjoint-batch", type=int, default=None, metavar="SCENES",
                    help="print the batched adjoint summary alone, on the first SCENES scenes, over --steps steps")
    ap.add_argument("--particles", type=int, default=None,
                    help="particle count of the generated scene (profiling captures of a smaller case)")
    ap.add_argument("--single", action="store_true",
                    help="headline precision only: no second precision, e2e, error or CPU legs (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: start the ranks here, as the multi-GPU
        # launcher would (rank 0 prints the line)
        import socket
        with socket.socket() as sock:
            sock.bind(("127.0.0.1", 0))
            port = sock.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr=127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *sys.argv[1:]]
        sys.exit(subprocess.call(cmd))
    if world != args.gpus and args.impl != "reference":
        ap.error(f"--gpus {args.gpus} but WORLD_SIZE={world}")
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.adjoint_only or args.adjoint_batch or args.adjoint_c4:
        from dem_mbd_cuda_gb300 import build as _b
        _b.build()
        if args.adjoint_c4:
            print(json.dumps(c4_adjoint_summary()))
        elif args.adjoint_batch:
            print(json.dumps(batch_adjoint_summary(args.adjoint_batch, args.steps, min(10, args.steps))))
        else:
            print(json.dumps(adjoint_summary()))
        return
    if args.impl == "reference" and rank != 0:
        return
    scene, desc = make_scene(args.config, args.particles)
    if isinstance(scene, list) and not args.single:
        ap.error("--config c4 runs with --single; the default line carries it as batch_256")
    n_all = sum(sc.n for sc in scene) if isinstance(scene, list) else scene.n
    sharded = isinstance(scene, list) and world > 1 and args.impl != "reference"
    if sharded:
        # a batch shards by scene: each rank runs its share as one engine
        from dem_mbd_cuda_gb300.shard import partition
        parts = partition([sc.n for sc in scene], world)
        scene = [scene[i] for i in parts[rank]]

    if args.impl == "reference":
        # The reference's hot path is CUDA-only; its CPU implementation of the
        # path here is the oracle port on all host cores.  A CPU step of the
        # 2M-sphere drum takes about half a second, so the timed steps are
        # bounded to about a minute of work (the line states how many ran).
        from oracle import oracle as orc
        orc.build()
        from oracle.oracle import Oracle
        threads = os.cpu_count() or 1
        o = Oracle(scene, threads=threads)
        o.run(1)
        t0 = time.perf_counter()
        warm = 1
        while warm < args.warmup and time.perf_counter() - t0 < 10.0:
            o.run(1)
            warm += 1
        done = 0
        t0 = time.perf_counter()
        while done < args.steps:
            o.run(1)
            done += 1
            if time.perf_counter() - t0 >= 60.0:
                break
        dt = time.perf_counter() - t0
        v = scene.n * done / dt
        line = {"impl": "reference", "metric": "particle-steps/s", "value": v, "unit": "particle-steps/s",
                "n_gpus": 0, "steps": done, "warmup": warm, "ms_per_step": dt * 1000 / done,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": desc, "particles": scene.n, "triangles": scene.n_triangles},
                "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                                 "sample": f"{done} of the {args.steps} requested steps of the workload (at most "
                                           f"60 s of work) after {warm} warm-up steps"},
                "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        # one GPU per rank, fixed before the first CUDA call (the engine runs
        # on the current device): this rank's entry of the visible list, or
        # its local rank when no list is set; a list of one was already
        # narrowed by the launcher
        ids = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        if len(ids) > 1:
            if local >= len(ids):
                raise SystemExit(f"local rank {local} has no GPU in CUDA_VISIBLE_DEVICES={','.join(ids)}")
            os.environ["CUDA_VISIBLE_DEVICES"] = ids[local]
        elif not ids:
            os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    from dem_mbd_cuda_gb300 import build
    build.build()
    if dist:
        dist.barrier()
    e, ms, clocks, stats, phases, after = run_engine(scene, args.precision, args.steps, args.warmup)
    nlists = after["neighbor_lists"]
    if args.single:
        if dist:
            from dem_mbd_cuda_gb300.shard import max_over_ranks
            ms = max_over_ranks(ms)
        # sharded: the whole batch's particles over the slowest rank's time;
        # replicas: every rank's particles over the slowest rank's time
        value = (n_all if sharded else world * n_all) * args.steps / (ms / 1000.0)
        if rank != 0:
            return
        print(json.dumps({"metric": "particle-steps/s", "value": value, "ms_per_step": ms / args.steps,
                          "n_gpus": world, "scaling": "strong" if sharded else "weak",
                          "parallelism": ("scenes sharded over %d ranks" % world) if sharded
                          else ("replicas" if world > 1 else "single"),
                          "precision": args.precision, "phase_ms": dict(zip(PHASES, phases)),
                          "contact_sides_per_step": stats["particle_contacts"], "clocks": clocks}))
        return
    per_step_ms = ms / args.steps
    roof = roofline(phases, scene, stats, nlists, args.precision, e, per_step_ms, args.config)
    del e
    other = "fp64" if args.precision == "mixed" else "mixed"
    e_o, ms_o, _, _, phases_o, _ = run_engine(scene, other, args.steps, args.warmup)
    del e_o
    fp64_roof = fp64_roofline(phases_o if other == "fp64" else phases, args.config, "fp64")
    fp64_roof.update(fp64_roofline(phases, args.config, args.precision))
    if dist:
        t = __import__("torch").tensor([ms, ms_o], dtype=__import__("torch").float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, ms_o = float(t[0]), float(t[1])
    per_step_ms = ms / args.steps
    value = world * scene.n * args.steps / (ms / 1000.0)
    value_other = world * scene.n * args.steps / (ms_o / 1000.0)
    e2e_ms = e2e_run(scene, args.precision, args.steps, args.warmup)
    if dist:
        from dem_mbd_cuda_gb300.shard import max_over_ranks
        e2e_ms = max_over_ranks(e2e_ms)
    e2e_value = world * scene.n * args.steps / (e2e_ms / 1000.0)
    if rank != 0:
        return
    errs = load_error(scene)
    contacts = stats["particle_contacts"]
    cpu = None
    if not args.no_cpu_baseline:
        v, cores, done, dt = cpu_baseline(scene)
        cpu = {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": "port",
               "sample": f"{done} steps of the same workload on {cores} threads ({dt:.1f} s)"}
    subs = {}
    if args.config != "c2" and not args.no_drum:
        subs["drum_2m"] = scene_summary("c2", args.steps, args.warmup)
    if args.config != "c1" and not args.no_c1:
        subs["c1_200k"] = scene_summary("c1", args.steps, args.warmup)
    if args.config != "c4" and not args.no_batch:
        subs["batch_256"] = batch_summary(args.steps, args.warmup)
    if not args.no_reference_cuda:
        ref = reference_cuda_summary([args.config] + (["c1"] if args.config != "c1" and not args.no_c1 else []),
                                     args.steps, args.warmup)
        if args.config in ref:
            ref[args.config]["engine_over_reference"] = {
                args.precision: value / world / ref[args.config]["value"],
                other: value_other / world / ref[args.config]["value"]}
        if "c1" in ref and "c1_200k" in subs:
            ref["c1"]["engine_over_reference"] = {p: subs["c1_200k"][p]["value"] / ref["c1"]["value"]
                                                  for p in ("mixed", "fp64")}
        subs["reference_fp64_cuda"] = ref
    if not args.no_adjoint:
        subs["adjoint_c3"] = adjoint_summary()
        if not args.no_batch:
            subs["adjoint_batch"] = batch_adjoint_summary()
            subs["calibration_c4"] = calibration_summary()
            subs["adjoint_c4"] = c4_adjoint_summary()
    if not args.no_autotune:
        subs["autotuned"] = autotune_summary(scene, args.precision)
    nb = scene.n_bodies
    line = {
        "metric": "particle-steps/s",
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": per_step_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-contact/f64-state" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": desc, "particles": scene.n, "triangles": scene.n_triangles, "precision": args.precision,
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "per-step working set (state, records, history, contact list) exceeds the 129 MB L2"},
        "fp64_value" if args.precision == "mixed" else "mixed_value": value_other,
        "contacts_per_s": contacts * args.steps / (ms / 1000.0) / 2,
        "contact_sides_per_step": contacts,
        "body_manifolds_per_step": stats["body_contacts"],
        "load_error_vs_fp64": errs,
        "phase_ms": dict(zip(PHASES, phases)),
        "phase_ms_" + other: dict(zip(PHASES, phases_o)),
        "neighbor_lists": nlists,
        "roofline": roof,
        "fp64_roofline": fp64_roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": 13 * 8 * nb,
                "d2h_bytes_per_step": 38 * 8 * nb + 16 * 4},
        "gpu_launches": launches_per_step(scene) * args.steps,
        "clocks": clocks,
    }
    line.update(subs)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
