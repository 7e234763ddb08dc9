#!/usr/bin/env python3
"""Benchmark of the batched hydrodynamic wrench step on GB300.

Workload (default ``batch``): 4096 rigid bodies with distinct meshes drawn
from icospheres (320-20480 faces), subdivided boxes (12-49152 faces) and
capped cylinders 1.6 m x 0.2 m (500-50000 faces), about 37M faces in total;
CG depth U(-1.0,+0.3) m, uniform random orientation, v ~ U(-1,1)^3 m/s,
omega ~ U(-0.5,0.5)^3 rad/s, flat surface, uniform current (0.2,0,0) m/s,
rho = 1025 kg/m^3.  Synthetic, seeded data.

One step = one evaluation of every body's wrench (the per-body loop of the
hydrodynamics block of Stonefish's SimulationManager::SimulationTickCallback)
with the inputs resident in HBM (``value``), and through the host-buffer C ABI
call with the host<->device copies inside the timed region (``e2e``).  The
mesh data (~0.5 GB) is larger than L2, so no flush is needed between steps.

``--impl reference`` times the reference's own routine on the host cores
on the same workload: its hydrodynamics functions compiled from its sources
(oracle/_ref) where they were built on this machine, else the oracle's REF32
restatement (FP32 glm-order face arithmetic); one task per body on all host
threads either way.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "hydro wrench evals/s & faces/s, 1 GB300: exact FP32 vs surrogate at stated error"
UNIT = "wrench evals/s"
BYTES_PER_FACE = 18.0      # indexed mesh: 12 B of indices + 0.5 x 12 B of positions


from stonefish_gb300.replicas import max_over_ranks, whole_job_rate  # noqa: E402


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines: list[str] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
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
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "power_w_max": float(max(power)), "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------- helpers
def measured_peaks() -> tuple[float, str]:
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(workload: str):
    """DRAM bytes per launch of the chunk kernel from the committed ncu summary."""
    p = os.path.join(HERE, "profiles", f"chunk_kernel_{workload}.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_full_launch:"):
            return float(line.split(":")[1].split()[0])
    return None


def profile_instructions(workload: str):
    """Warp instructions the chunk kernel executes per processed face, from
    the committed ncu summary (smsp__inst_executed.sum of one launch over its
    processed faces), or None."""
    p = os.path.join(HERE, "profiles", f"chunk_kernel_{workload}.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("warp_instructions_per_processed_face:"):
            return float(line.split(":")[1].split()[0])
    return None


ISSUE_PER_SM_CLOCK = 4     # four SM sub-partitions, each issuing one warp instruction per clock


def issue_roofline(workload: str, processed_faces: int, kernel_s: float, sm_mhz) -> dict | None:
    """The chunk kernel against the SMs' instruction-issue rate: its warp
    instructions per launch (ncu count per processed face x processed faces)
    over its CUDA-event time, against SMs x 4 issue slots x the SM clock
    sampled during the run.  For the shared-mesh workloads (one hull, mesh
    and wave grid in L2) this, not HBM, is the bound; for the distinct-mesh
    batch it is the bound the kernel is nearer to."""
    import torch
    ipf = profile_instructions(workload)
    if ipf is None or not sm_mhz or kernel_s <= 0:
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    achieved = ipf * processed_faces / kernel_s
    peak = sms * ISSUE_PER_SM_CLOCK * sm_mhz * 1e6
    return {"bound": "issue", "achieved": achieved, "peak": peak, "unit": "warp instructions/s",
            "frac": achieved / peak, "instructions_per_face": ipf, "sm_mhz": sm_mhz, "sms": sms,
            "rule": "ncu smsp__inst_executed.sum per processed face (profiles/chunk_kernel_<workload>.txt) x "
                    "processed faces / chunk-kernel time; peak = SMs x 4 warp instructions per clock x "
                    "median SM clock under load"}


def hull_states_workload(faces: int, n_bodies: int, seed: int = 505):
    """The surrogate's torpedo hull (``faces`` faces) at n seeded states over
    the wave field, as an exact-step workload (the CPU reference arm of the
    surrogate and rollout lines)."""
    from stonefish_gb300 import scenarios
    from stonefish_gb300 import surrogate as S
    xyz, fc = S.hull_mesh(faces)
    bodies = S.sample_states(np.random.default_rng(seed), n_bodies)
    return {"meshes": [(xyz, fc)], "bodies": bodies, "ocean": S.wave_ocean(), "waves": scenarios.wave_grid()}


def build_workload(name: str, n_bodies: int | None):
    from stonefish_gb300 import scenarios
    if name == "surrogate":
        return hull_states_workload(12000, n_bodies or 512)
    if name == "rollout":
        return hull_states_workload(8000, n_bodies or 512)
    if name == "batch":
        return scenarios.mixed_batch(n_bodies=n_bodies or 4096)
    if name == "waves":
        return scenarios.torpedo_waves(n_bodies=n_bodies or 1024)
    if name == "sphere":
        return scenarios.single_sphere(steps=n_bodies or 1000)
    raise SystemExit(f"unknown workload {name}")


def workload_config(name: str, sc) -> dict:
    nf = int(sum(len(f) for _, f in sc["meshes"]))
    per_body_faces = np.array([len(sc["meshes"][m][1]) for m in sc["bodies"]["mesh"]])
    cfg = {"workload": {"batch": "mixed_batch_4096_bodies_distinct_meshes",
                        "waves": "torpedo_hulls_on_1024x1024_wave_grid",
                        "sphere": "single_icosphere_1280_faces_1000_states",
                        "surrogate": "exact step on the 12000-face torpedo, seeded states over the wave grid",
                        "rollout": "exact step on the 8000-face torpedo, seeded states over the wave grid"}[name],
           "bodies": int(len(sc["bodies"])), "faces_per_step": int(per_body_faces.sum()),
           "distinct_mesh_faces": nf, "surface": "waves" if sc["ocean"].waves else "flat",
           "current_mps": [0.2, 0.0, 0.0], "density": 1025.0,
           "l2_policy": "inputs larger than L2 (mesh data > 129 MB)" if nf * 13 > 2e8
           else "inputs L2-resident (shared mesh)"}
    return cfg, per_body_faces


def cpu_implementation():
    """The CPU implementation the CPU legs time.  Where the reference's own
    hydrodynamics functions were compiled from its sources on this machine
    (oracle/_ref), those; else the oracle's REF32 restatement (the
    reference's arithmetic).  Both run one task per body on a thread pool, as
    SimulationManager.cpp:1620-1655 does.  Returns (run, kind, what) where
    run(threads, workload, io) runs one step and returns its seconds."""
    from stonefish_gb300 import scenarios
    st = scenarios.settings()
    try:
        from oracle.ref import Reference
        if Reference.available():
            r = Reference()
            return ((lambda threads, sc, io: r.batch(threads, sc["bodies"], sc["meshes"], sc["ocean"], st, io,
                                                     waves=sc.get("waves"))),
                    "reference", "the reference's SolidEntity hydrodynamics compiled from its sources, "
                                 "one task per body")
    except (OSError, RuntimeError):
        pass
    from oracle import REF32, Oracle
    o = Oracle()
    return ((lambda threads, sc, io: o.batch(REF32, threads, sc["bodies"], sc["meshes"], sc["ocean"], st, io,
                                             waves=sc.get("waves"))),
            "port", "REF32 oracle restatement of the reference's arithmetic, one task per body "
                    "(the reference's sources are not on this machine)")


def cpu_baseline(sc, threads: int, budget_s: float = 12.0, max_steps: int = 20):
    """Median seconds of full steps of the workload on host threads."""
    from stonefish_gb300 import scenarios
    run, kind, what = cpu_implementation()
    io = scenarios.new_wrenches(len(sc["bodies"]))
    times = []
    t_start = time.perf_counter()
    while len(times) < max_steps and (time.perf_counter() - t_start) < budget_s:
        times.append(run(threads, sc, io))
    return float(np.median(times)), len(times), kind, what


def _pair_scaled(a, c, bodies) -> np.ndarray:
    """Per-body worst pair-scaled error of wrenches a against c: forces over
    the body's force scale S = max(|Fb|, |Fdq|, |Fdf|) of c, torques over S
    times the body's half AABB diagonal."""
    S = np.maximum(np.max(np.stack([np.linalg.norm(c[k], axis=1) for k in ("Fb", "Fdq", "Fdf")]), axis=0), 1e-300)
    L = 0.5 * np.linalg.norm(bodies["aabb_max"] - bodies["aabb_min"], axis=1)
    errs = [np.linalg.norm(a[k] - c[k], axis=1) / S for k in ("Fb", "Fdq", "Fdf")]
    errs += [np.linalg.norm(a[k] - c[k], axis=1) / (S * L) for k in ("Tb", "Tdq", "Tdf")]
    return np.max(np.stack(errs), axis=0)


def fp64_error(sc, gpu_io, frame: str) -> dict:
    """The GPU result against the all-FP64 evaluation on every body with a
    face loop, next to the reference's own FP32 arithmetic (REF32) on the
    same bodies; and the GPU against the oracle variant with its own
    arithmetic (MIRROR32: the reference's FP32 faces with FP64 sums, on the
    bodies moved to the origin for the centred frame)."""
    from oracle import MIRROR32, REF32, REF64, Oracle
    from oracle.oracle import centred_scene
    from stonefish_gb300 import abi, scenarios
    act = (gpu_io["position"] == abi.CROSSING_SURFACE) | (gpu_io["position"] == abi.INSIDE)
    if not act.any():
        return {}
    o = Oracle()
    threads = os.cpu_count() or 1
    st = scenarios.settings()
    b = sc["bodies"]
    out = {}
    for tag, var, bodies in (("ref64", REF64, b), ("ref32", REF32, b),
                             ("mirror", MIRROR32, centred_scene(b) if frame == "centred" else b)):
        io = scenarios.new_wrenches(len(b))
        o.batch(var, threads, bodies, sc["meshes"], sc["ocean"], st, io, waves=sc.get("waves"))
        out[tag] = io

    def stats(e):
        e = e[act]
        return {"median": float(np.median(e)), "p99": float(np.percentile(e, 99)), "max": float(e.max()),
                "frac_le_1e-5": float(np.mean(e <= 1e-5))}
    res = {"metric": "pair-scaled |x-x64| / force scale (torques / force scale x size), every active body",
           "frame": frame, "bodies": int(act.sum())}
    res.update(stats(_pair_scaled(gpu_io, out["ref64"], b)))
    res["reference_fp32_vs_fp64"] = stats(_pair_scaled(out["ref32"], out["ref64"], b))
    if sc.get("waves") is None or frame == "world":
        m = _pair_scaled(gpu_io, out["mirror"], b)[act]
        res["parity_vs_own_arithmetic"] = {"oracle": "MIRROR32" + (" on centred bodies" if frame == "centred" else ""),
                                          "max": float(m.max()), "positions_equal":
                                          bool(np.array_equal(gpu_io["position"], out["mirror"]["position"]))}
    return res


# ------------------------------------------------------------- surrogate
MLP_FLOP_PER_EVAL = 2.0 * (16 * 256 + 256 * 256 + 256 * 256 + 256 * 6)   # unpadded 16-256-256-256-6


def measured_tensor_peak() -> tuple[float, str]:
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def surrogate_bench(args, device: int) -> dict:
    """The learned wrench surrogate on the 12000-face torpedo hull over the
    wave field: label ``--sur-train`` states with the exact step (FP64 cut
    points), train the MLP with the library's kernels, then time gated
    inference over batches of 65536 states against the exact FP32 step on
    the same states.  Eight distinct state batches (240 MB of body records,
    more than L2) are cycled through the timed steps."""
    import torch

    from stonefish_gb300 import abi, scenarios
    from stonefish_gb300 import surrogate as S
    from stonefish_gb300.hydro import HydroContext

    t_setup = time.perf_counter()
    h64 = HydroContext(device, cut_precision=abi.CUT_FP64)
    h32 = HydroContext(device)
    xyz, fc = S.hull_mesh()
    waves = scenarios.wave_grid()
    m64, m32 = h64.upload_mesh(xyz, fc), h32.upload_mesh(xyz, fc)
    h64.set_wave_grid(waves)
    h32.set_wave_grid(waves)
    ocean, st = S.wave_ocean(), scenarios.settings()
    lab = S.Labeller(h64, m64, ocean, st)
    t0 = time.perf_counter()
    F, T = S.generate(lab, args.sur_train, seed=101)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    fs_, ts_ = S.hull_scales(ocean)
    # two networks of the same hull (different seeds), targets scaled as the
    # wrench metric weighs them
    sur = S.Surrogate(h32, batch=args.sur_batch, seed=0)
    sur.fit_normalisation(F, T, target_scales=(fs_, ts_))
    info = sur.fit(F, T, epochs=args.sur_epochs, lr=args.sur_lr)
    sur2 = S.Surrogate(h32, batch=args.sur_batch, seed=1)
    sur2.fit_normalisation(F, T, target_scales=(fs_, ts_))
    info2 = sur2.fit(F, T, epochs=args.sur_epochs, lr=args.sur_lr)
    del F, T
    nB, n_sets = 65536, 8
    # the ensemble gate's threshold, from held-out labelled states (not the
    # evaluation states below)
    cal = S.sample_states(np.random.default_rng(303), nB)
    Fc = torch.empty((nB, 16), dtype=torch.float32, device="cuda")
    Tc = torch.empty((nB, 6), dtype=torch.float32, device="cuda")
    Wc = torch.zeros(nB * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    lab.label(cal, Fc, Tc, wrenches=Wc)
    zc = torch.zeros((nB, 16), dtype=torch.float32, device="cuda")
    pa = sur.infer_tc(Fc, zc, sur.tc_weights())[:, :6].cpu().numpy()
    pb = sur2.infer_tc(Fc, zc, sur2.tc_weights())[:, :6].cpu().numpy()
    cal_in = Wc.cpu().numpy().view(abi.WRENCH_DTYPE)["position"] != abi.INSIDE
    if not args.sur_gate_inside:
        cal_in = np.ones(nB, dtype=bool)   # INSIDE states are admitted too: calibrate on all of them
    # calibrated for 0.95% on the held-out states: 5% of margin below the 1%
    # bar for the difference between two samples of 65,536 states
    calib = S.calibrate_disagreement(pa, pb, Tc.cpu().numpy(), cal_in, ocean, target_p99=0.0095, max_reject=0.04)
    del Fc, Tc, Wc, zc
    rng = np.random.default_rng(202)
    sets, d_sets = [], []
    for _ in range(n_sets):
        b = S.sample_states(rng, nB)
        b["mesh"] = m32
        sets.append(b)
        d_sets.append(torch.from_numpy(np.frombuffer(b.tobytes(), dtype=np.uint8).copy()).cuda())
    Ft = torch.empty((nB, 16), dtype=torch.float32, device="cuda")
    Tt = torch.empty((nB, 6), dtype=torch.float32, device="cuda")
    Wt = torch.zeros(nB * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    lab.label(sets[0], Ft, Tt, wrenches=Wt)
    inside = Wt.cpu().numpy().view(abi.WRENCH_DTYPE)["position"] == abi.INSIDE
    del Wt
    # the network alone, for comparison
    z1 = torch.zeros((nB, 16), dtype=torch.float32, device="cuda")
    single = S.wrench_errors(sur.infer_tc(Ft, z1, sur.tc_weights())[:, :6].cpu().numpy(), Tt.cpu().numpy(), ocean)
    del z1
    # the two networks' mean on the states in the reference's INSIDE regime
    # (analytic buoyancy), whatever the gates decide
    z2 = torch.zeros((nB, 16), dtype=torch.float32, device="cuda")
    mean2 = 0.5 * (sur.infer_tc(Ft, z2, sur.tc_weights())[:, :6].cpu().numpy() +
                   sur2.infer_tc(Ft, z2, sur2.tc_weights())[:, :6].cpu().numpy())
    del z2
    err_inside = S.wrench_errors(mean2[inside], Tt.cpu().numpy()[inside], ocean) if inside.any() else {}
    gp = S.GatedPredictor(sur, h32, m32, nB, ocean, st, second=sur2, tau=calib["tau"],
                          gate_inside=bool(args.sur_gate_inside), audit_stride=1024)
    out = gp.predict(d_sets[0]).cpu().numpy()
    adm = gp.admitted()
    err = S.wrench_errors(out, Tt.cpu().numpy(), ocean)
    err_adm = S.wrench_errors(out[adm], Tt.cpu().numpy()[adm], ocean)
    rejected = gp.rejected()
    setup_s = time.perf_counter() - t_setup

    steps = max(8, min(args.steps, 400))
    stream = torch.cuda.current_stream()
    for i in range(max(args.warmup, 3)):
        gp.predict(d_sets[i % n_sets])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        gp.predict(d_sets[i % n_sets])
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # the network alone (the fused tcgen05 kernel predict() launches), for
    # the tensor-core roofline; and the four mma.sync GEMMs for comparison
    feats_d = gp.bufs["feats"]
    for _ in range(3):
        sur.infer_tc(feats_d, gp.z16, gp.tcw)
    e0.record(stream)
    for _ in range(steps):
        sur.infer_tc(feats_d, gp.z16, gp.tcw)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_mlp = e0.elapsed_time(e1) / steps
    bufs = sur._infer_bufs(nB)
    for _ in range(3):
        sur._mlp(bufs, nB)
    e0.record(stream)
    for _ in range(steps):
        sur._mlp(bufs, nB)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_mma = e0.elapsed_time(e1) / steps
    # the exact FP32 step on the same states
    bx = h32.batch(np.full(nB, m32, dtype=np.uint32))
    io = torch.zeros(nB * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    sp = stream.cuda_stream
    for i in range(2):
        bx.compute_device(d_sets[i].data_ptr(), ocean, st, io.data_ptr(), sp)
    torch.cuda.synchronize()
    ex_steps = 4
    e0.record(stream)
    for i in range(ex_steps):
        bx.compute_device(d_sets[i % n_sets].data_ptr(), ocean, st, io.data_ptr(), sp)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_exact = e0.elapsed_time(e1) / ex_steps
    # end to end: pinned host states in, body-frame wrenches out
    # (predict() reads the page-locked states in place: the kernels fetch them
    # over the host link every step)
    h_in = torch.from_numpy(np.frombuffer(sets[0].tobytes(), dtype=np.uint8).copy()).pin_memory()
    h_out = torch.empty((nB, 6), dtype=torch.float32).pin_memory()
    e2e_steps = max(4, steps // 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h_out.copy_(gp.predict(h_in), non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    audit = gp.audit_errors()
    peak, kind = measured_tensor_peak()
    achieved = MLP_FLOP_PER_EVAL * nB / (ms_mlp / 1e3) / 1e12
    res = {
        "value": nB / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "states_per_step": nB,
        "workload": "torpedo_12000_faces_on_1024x1024_wave_grid, 65536 states per step",
        "exact_fp32_gpu": {"value": nB / (ms_exact / 1e3), "unit": UNIT, "ms_per_step": ms_exact,
                           "faces_per_s": nB * len(fc) / (ms_exact / 1e3)},
        "speedup_vs_exact_gpu": ms_exact / ms,
        "error": dict(err_adm, metric="|dF| / (rho g V), |dT| / (rho g V L/2); wrench = max of the two; "
                                      "against exact labels (FP32 faces, FP64 cut points and sums); "
                                      "states whose output is the network's (admitted by the gates)"),
        "error_all_outputs": dict(err, note="every state of the step; gated and audited states carry the "
                                            "exact step's wrench"),
        "error_single_network": dict(single, note="one network, no gates, same states"),
        "error_inside_states": dict(err_inside, frac=float(inside.mean()),
                                    note="the two networks' mean on the states whose fluid position is INSIDE "
                                         "(sent to the exact step when the INSIDE gate is on)"),
        "gate": {"rejected_frac": rejected / nB, "rules": "feature box + Mahalanobis radius; "
                 + ("fluid position INSIDE; " if args.sur_gate_inside else "") +
                 "the two networks' disagreement above tau (calibrated on 65536 held-out labelled "
                 "states for an admitted 99th percentile <= 0.0095, at most 4% rejected)", "calibration": calib},
        "audit": {"rows": int(audit.size), "stride": gp.audit_stride,
                  "median": float(np.median(audit)) if audit.size else None,
                  "p99": float(np.percentile(audit, 99)) if audit.size else None,
                  "max": float(audit.max()) if audit.size else None,
                  "note": "every predict() also runs every 1024th admitted state through the exact step "
                          "(its output becomes exact) and records the network's error there"},
        "gate_rejected_frac": rejected / nB,
        "train": {"samples": args.sur_train, "epochs": args.sur_epochs, "batch": args.sur_batch,
                  "networks": 2, "target_scaling": "force / (rho g V), torque / (rho g V L/2)",
                  "lr": args.sur_lr, "label_s": t_gen, "train_s": info["seconds"] + info2["seconds"],
                  "train_samples_per_s": info["samples_per_s"], "final_loss": info["loss"][-1]},
        "e2e": {"value": nB / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": int(nB * abi.BODY_DTYPE.itemsize),
                "d2h_bytes_per_step": int(nB * 6 * 4),
                "transfer": "the states stay in page-locked host memory and the kernels read them in "
                            "place every step (the features kernel reads the pose and velocity fields); "
                            "the 6 outputs per state are copied back"},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_source": kind, "traffic": None,
                     "kernel": "mlp_tc_kernel: the whole 16-256-256-256-6 network fused, tcgen05.mma "
                               "kind::f16 M128 with TMEM accumulators, weights by bulk copy",
                     "kernel_us": ms_mlp * 1e3,
                     "flop_rule": f"{MLP_FLOP_PER_EVAL:.0f} FLOP per state (unpadded layers)",
                     "mma_sync_gemms_us": ms_mma * 1e3,
                     "mma_sync_tflops": MLP_FLOP_PER_EVAL * nB / (ms_mma / 1e3) / 1e12},
        "gpu_launches_per_step": gp.launches,
        "setup_s": setup_s,
    }
    for o in (bx, gp, lab):
        o.close()
    h32.close()
    h64.close()
    return res


# --------------------------------------------------------------- rollout
def rollout_bench(args, device: int) -> dict:
    """16384 hulls (8000-face torpedo, 50 kg, four fixed body-frame thrusts
    U(-20,20) N) over the wave field, 1000 steps of dt = 0.01 s by
    semi-implicit Euler, captured as one CUDA graph per rollout: once with
    the exact step and once with the surrogate (trained here on the same
    hull) behind its gate.  Reports env-steps/s of each and how far the two
    trajectories drift apart."""
    import torch

    from stonefish_gb300 import abi, scenarios
    from stonefish_gb300 import rollout as RO
    from stonefish_gb300 import surrogate as S
    from stonefish_gb300.hydro import HydroContext

    n, steps, faces = args.roll_envs, args.roll_steps, 8000
    t_setup = time.perf_counter()
    h64 = HydroContext(device, cut_precision=abi.CUT_FP64)
    h32 = HydroContext(device)
    xyz, fc = S.hull_mesh(faces)
    waves = scenarios.wave_grid()
    m64, m32 = h64.upload_mesh(xyz, fc), h32.upload_mesh(xyz, fc)
    h64.set_wave_grid(waves)
    h32.set_wave_grid(waves)
    ocean, st = S.wave_ocean(), scenarios.settings()
    lab = S.Labeller(h64, m64, ocean, st)
    surf = RO.surface_z(h32, ocean)
    # training envelope of the floating hulls: CG within 0.6 m below to 0.5 m
    # above the local surface, |v| components to 3 m/s, body-frame rates to
    # 10 rad/s about the long axis (roll has no restoring moment and little
    # inertia, so hulls spin up) and 2.5 rad/s about the others (the pitch
    # oscillation reaches rates above 1 rad/s)
    F, T = S.generate(lab, args.roll_train, seed=303, depth=(-0.5, 0.6), v_range=3.0, w_body=(10.0, 2.5, 2.5),
                      surface=surf)
    # two networks, their mean as the wrench; the roll torque is weighed 10
    # times the others: a circular hull has no restoring moment in roll and
    # 1.56 kg m^2 of inertia about its axis, so an error of 0.1% of the torque
    # scale (rho g V L/2, ~5.8 kN m) would spin it up within a second
    fs_, ts_ = S.hull_scales(ocean)
    nets = []
    for seed in (0, 1):
        net = S.Surrogate(h32, batch=args.sur_batch, seed=seed)
        net.fit_normalisation(F, T, target_scales=(fs_, fs_, fs_, ts_ / 10.0, ts_, ts_))
        net.fit(F, T, epochs=args.sur_epochs, lr=args.sur_lr)
        nets.append(net)
    sur, sur2 = nets
    del F, T
    lab.close()
    init = RO.initial_states(np.random.default_rng(404), n, surface=surf)
    ex = RO.Rollout(h32, m32, n, ocean, st, "exact")
    ex.reset(init)
    k_ex = ex.capture(steps)
    gp = S.GatedPredictor(sur, h32, m32, n, ocean, st, second=sur2)
    su = RO.Rollout(h32, m32, n, ocean, st, "surrogate", predictor=gp)
    su.reset(init)
    k_su = su.capture(steps)
    # the same exact rollout with FP64 cut points: how far two exact
    # evaluations that differ only in rounding drift apart (chaos floor)
    e64 = RO.Rollout(h64, m64, n, ocean, st, "exact")
    e64.reset(init)
    k_64 = e64.capture(steps)
    setup_s = time.perf_counter() - t_setup
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res = {}
    clocks = {}
    for name, ro, k in (("exact", ex, k_ex), ("surrogate", su, k_su), ("exact_fp64_cut", e64, k_64)):
        ro.reset(init)
        torch.cuda.synchronize()
        sampler = ClockSampler(device)
        sampler.start()
        e0.record(stream)
        ro.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        clocks[name] = sampler.stop()
        ms = e0.elapsed_time(e1)
        res[name] = {"env_steps_per_s": n * steps / (ms / 1e3), "ms_per_step": ms / steps,
                     "rollout_s": ms / 1e3, "gpu_launches_per_step": k / steps, "clocks": clocks[name]}
        if name == "exact":
            # hulls with a face loop at the last step (not out of the water),
            # all of whose tiles the wave surface makes the kernel process
            pos = ro.io.cpu().numpy().view(abi.WRENCH_DTYPE)["position"]
            looping = int(np.count_nonzero((pos == abi.CROSSING_SURFACE) | (pos == abi.INSIDE)))
            res[name]["faces_processed_last_step"] = looping * faces
            # the whole step's time (rigid step, prep, finalize included)
            # against the chunk kernel's instruction count: a lower bound
            res[name]["issue_roofline"] = issue_roofline("waves", looping * faces, ms / steps / 1e3,
                                                         clocks[name].get("sm_mhz"))
    res["surrogate"]["gate_rejected_last_step"] = gp.rejected()
    a, b, c = ex.snapshots(), su.snapshots(), e64.snapshots()
    res["divergence"] = {f"step_{(i + 1) * 100}": RO.divergence(a[i], b[i], init) for i in range(len(a))}
    res["divergence_exact_fp32_vs_fp64_cut"] = {f"step_{(i + 1) * 100}": RO.divergence(a[i], c[i], init)
                                                for i in range(len(a))}
    res["exact"]["states"] = {f"step_{(i + 1) * 100}": RO.state_stats(a[i]) for i in range(len(a))}
    res["surrogate"]["states"] = {f"step_{(i + 1) * 100}": RO.state_stats(b[i]) for i in range(len(b))}
    res["finite"] = bool(all(np.all(np.isfinite(r.host_states()["p"])) for r in (ex, su, e64)))
    res["speedup_surrogate_vs_exact"] = res["exact"]["rollout_s"] / res["surrogate"]["rollout_s"]
    res["workload"] = (f"{n} torpedo hulls x {faces} faces, 50 kg, 4 thrusters U(-20,20) N, dt 0.01 s, "
                       f"{steps} steps in one CUDA graph, 1024x1024 wave grid; surrogate: mean of two "
                       f"networks trained on {args.roll_train} exact-labelled states of the same hull")
    res["setup_s"] = setup_s
    for o in (ex, su, gp, e64):
        o.close()
    h32.close()
    h64.close()
    return res


def section_line(args, rank: int, world: int, local_rank: int, dist):
    """``--workload surrogate|rollout``: that section alone, as the line's
    headline (one replica per rank; rank 0 reports its own replica)."""
    if args.workload == "surrogate":
        sec = surrogate_bench(args, local_rank)
        value, unit, ms = sec["value"], UNIT, sec["ms_per_step"]
        launches, e2e = sec["gpu_launches_per_step"], sec["e2e"]
        roof = sec["roofline"]
        cfg = {"workload": sec["workload"], "states_per_step": sec["states_per_step"]}
        dtype = "bf16 MLP (fp32 accumulate), f32 exact fallback"
    else:
        sec = rollout_bench(args, local_rank)
        value, unit = sec["surrogate"]["env_steps_per_s"], "env-steps/s"
        ms = sec["surrogate"]["ms_per_step"]
        launches = sec["surrogate"]["gpu_launches_per_step"]
        e2e = None
        roof = sec["exact"].get("issue_roofline")
        cfg = {"workload": sec["workload"]}
        dtype = "f64 rigid state, f32 faces / bf16 MLP wrench"
    if rank != 0:
        return None
    return {"metric": METRIC, "value": value * world, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded states)",
            "config": dict(cfg, parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
            "e2e": e2e, "roofline": roof, "gpu_launches": launches * args.steps, args.workload: sec}


# ---------------------------------------------------------------- GPU arm
def run_gpu(args, rank: int, world: int, local_rank: int, dist):
    import torch

    from stonefish_gb300 import abi, scenarios
    from stonefish_gb300.hydro import HydroContext

    torch.cuda.set_device(local_rank)
    if args.workload in ("surrogate", "rollout"):
        return section_line(args, rank, world, local_rank, dist)
    t0 = time.perf_counter()
    sc = build_workload(args.workload, args.n_bodies)
    cfg, per_body_faces = workload_config(args.workload, sc)
    log(f"[rank {rank}] workload built in {time.perf_counter() - t0:.1f}s: {cfg}")
    h = HydroContext(device=local_rank, cut_precision=abi.CUT_FP32 if args.cut == "fp32" else abi.CUT_FP64,
                     tile_faces=args.chunk_faces, ctas_per_sm=args.ctas_per_sm,
                     frame=abi.FRAME_CENTRED if args.frame == "centred" else abi.FRAME_WORLD)
    t0 = time.perf_counter()
    if sc.get("waves") is not None:
        h.set_wave_grid(sc["waves"])
    ids = np.array([h.upload_mesh(x, f) for x, f in sc["meshes"]], dtype=np.uint32)
    log(f"[rank {rank}] meshes uploaded in {time.perf_counter() - t0:.1f}s")
    bodies = sc["bodies"].copy()
    bodies["mesh"] = ids[sc["bodies"]["mesh"]]
    batch = h.batch(bodies["mesh"])
    settings = scenarios.settings()
    ocean = sc["ocean"]
    nb = len(bodies)

    d_bodies = torch.from_numpy(bodies.view(np.uint8).copy()).cuda()
    d_io = torch.zeros(nb * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream

    def step():
        batch.compute_device(d_bodies.data_ptr(), ocean, settings, d_io.data_ptr(), sptr)

    tune = None
    if not args.no_autotune:
        d_scratch = torch.zeros_like(d_io)
        tune = batch.autotune(d_bodies.data_ptr(), ocean, settings, d_scratch.data_ptr(), sptr, reps=5)
        del d_scratch
        log(f"[rank {rank}] autotune: {tune}")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    graph = None
    if not args.no_graph:
        # the whole step (three kernels) as one CUDA graph, replayed per step
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            step()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                graph.replay()
        torch.cuda.synchronize()

    def timed_step():
        if graph is not None:
            graph.replay()
        else:
            step()

    gpu_io = d_io.cpu().numpy().view(abi.WRENCH_DTYPE).copy()
    active = (gpu_io["position"] == abi.CROSSING_SURFACE) | (gpu_io["position"] == abi.INSIDE)
    processed_faces = int(per_body_faces[active].sum())

    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.2)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    with torch.cuda.stream(stream):
        for _ in range(args.steps):
            timed_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    ms_per_step = ms / args.steps
    value = whole_job_rate(nb * args.steps, world, ms / 1e3)
    faces_per_s = whole_job_rate(int(per_body_faces.sum()) * args.steps, world, ms / 1e3)

    # end to end through the host-buffer call, pinned host memory
    h_bodies = torch.from_numpy(bodies.view(np.uint8).copy()).pin_memory()
    h_io = torch.zeros(nb * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    for _ in range(args.warmup):
        batch.compute_ptr(h_bodies.data_ptr(), ocean, settings, h_io.data_ptr())
    if dist is not None:
        dist.barrier()
    e2e_steps = max(1, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.compute_ptr(h_bodies.data_ptr(), ocean, settings, h_io.data_ptr())
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e_value = whole_job_rate(nb * e2e_steps, world, e2e_s)
    host_io = h_io.numpy().view(abi.WRENCH_DTYPE)
    assert host_io.tobytes() == gpu_io.tobytes(), "host-buffer and device-buffer results differ"

    # per-kernel device times: events the library records around its three
    # kernels on the launching stream, one step at a time (not graph-replayed)
    batch.profile(True)
    kt = {"prep": [], "chunk": [], "finalize": []}
    with torch.cuda.stream(stream):
        for i in range(min(args.steps, 200) + 3):
            step()
            t = batch.kernel_ms()
            if i >= 3:
                for k in kt:
                    kt[k].append(t[k])
    batch.profile(False)
    kernel_ms = {k: float(np.mean(v)) for k, v in kt.items()}

    if rank != 0:
        return None
    peak, peak_kind = measured_peaks()
    alg_bytes = BYTES_PER_FACE * processed_faces
    achieved = alg_bytes / (kernel_ms["chunk"] / 1e3) / 1e9
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 faces, f64 sums",
        "data": "synthetic (seeded meshes, poses and velocities)",
        "config": dict(cfg, processed_faces_per_step=processed_faces,
                       parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
        "faces_per_s": faces_per_s,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(nb * (abi.BODY_DTYPE.itemsize + abi.WRENCH_DTYPE.itemsize)),
                "d2h_bytes_per_step": int(nb * abi.WRENCH_DTYPE.itemsize), "steps": e2e_steps,
                "transfer": "hydro_batch_compute on page-locked host buffers: every step the per-body "
                            "kernels read the bodies and in-out wrenches from host memory and write the "
                            "wrenches back over the host link (no staging copies)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": profile_traffic(args.workload),
                     "kernel": "chunk_kernel (the face loop)",
                     "kernel_ms": kernel_ms["chunk"],
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "bytes_rule": "18 B per processed face (12 B of vertex indices + half of a 12 B "
                                   "FP32 vertex: a closed mesh has about half as many vertices as faces)",
                     "note": "the chunk kernel is issue-bound, not HBM-bound "
                             "(profiles/chunk_kernel_batch.txt)"},
        "issue_roofline": issue_roofline(args.workload, processed_faces, kernel_ms["chunk"] / 1e3,
                                         clocks.get("sm_mhz")),
        "kernel_ms": kernel_ms,
        "gpu_launches": args.steps * batch.last_launches(),
        "kernel_config": {"cut": args.cut, "frame": args.frame,
                          "chunk_faces": tune["chunk_faces"] if tune else (args.chunk_faces or 4096),
                          "ctas_per_sm": tune["ctas_per_sm"] if tune else (args.ctas_per_sm or 2),
                          "autotune": tune, "cuda_graph": graph is not None},
        "clocks": clocks,
    }
    if not args.no_error:
        result["error_vs_fp64"] = fp64_error(sc, gpu_io, args.frame)
    if not args.no_surrogate and world == 1:
        batch.close()
        result["surrogate"] = surrogate_bench(args, local_rank)
    if not args.no_rollout and world == 1:
        result["rollout"] = rollout_bench(args, local_rank)
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cpu_s, n, kind, what = cpu_baseline(sc, threads)
        cpu1_s, n1, _, _ = cpu_baseline(sc, 1, budget_s=5.0, max_steps=3)
        result["cpu_baseline"] = {"value": nb / cpu_s, "unit": UNIT, "cores": threads, "kind": kind,
                                  "sample": f"median of {n} full steps of the same workload ({what})",
                                  "faces_per_s": int(per_body_faces.sum()) / cpu_s,
                                  "value_1_thread": nb / cpu1_s,
                                  "sample_1_thread": f"median of {n1} full steps on one host thread"}
    batch.close()
    h.close()
    return result


def run_reference(args, rank: int):
    if rank != 0:
        return None
    sc = build_workload(args.workload, args.n_bodies)
    cfg, per_body_faces = workload_config(args.workload, sc)
    threads = os.cpu_count() or 1
    from stonefish_gb300 import scenarios
    run, kind, what = cpu_implementation()
    io = scenarios.new_wrenches(len(sc["bodies"]))
    # W warm-up steps (at most 5) and up to K timed steps, stopping early once
    # 60 s of CPU time are spent so the run stays within a few minutes
    warmup = max(1, min(args.warmup, 5))
    for _ in range(warmup):
        run(threads, sc, io)
    steps = 0
    total = 0.0
    while steps < max(1, args.steps) and (steps == 0 or total < 60.0):
        total += run(threads, sc, io)
        steps += 1
    nb = len(sc["bodies"])
    value = nb * steps / total
    unit = "env-steps/s" if args.workload == "rollout" else UNIT
    return {"metric": METRIC, "value": value, "unit": unit, "impl": "reference", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * total / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 faces (reference arithmetic)", "data": "synthetic", "config": cfg,
            "faces_per_s": int(per_body_faces.sum()) * steps / total,
            "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": kind,
                             "sample": f"{steps} full step{'s' if steps != 1 else ''} of the workload (at most --steps, "
                                       f"stopped after 60 s): {what}"},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "waves", "sphere", "surrogate", "rollout"])
    ap.add_argument("--n-bodies", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--cut", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--frame", default="centred", choices=["centred", "world"],
                    help="frame of the FP32 face arithmetic: centred on each body (default) or the "
                         "reference's world frame")
    ap.add_argument("--chunk-faces", type=int, default=0)
    ap.add_argument("--ctas-per-sm", type=int, default=0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-rollout", action="store_true")
    ap.add_argument("--roll-envs", type=int, default=16384)
    ap.add_argument("--roll-steps", type=int, default=1000)
    ap.add_argument("--roll-train", type=int, default=8_000_000)
    ap.add_argument("--sur-train", type=int, default=10_000_000)
    ap.add_argument("--sur-epochs", type=int, default=64)
    ap.add_argument("--sur-batch", type=int, default=4096)
    ap.add_argument("--sur-lr", type=float, default=3e-3)
    ap.add_argument("--sur-gate-inside", type=int, default=1, choices=[0, 1],
                    help="send states in the reference's INSIDE regime to the exact step (1, default) or "
                         "let the networks answer them (0)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if args.impl == "reference":
        res = run_reference(args, rank)
    else:
        if world > 1:
            import torch.distributed as dist_mod
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            import torch
            torch.cuda.set_device(local_rank)
            dist_mod.init_process_group("nccl")
            dist = dist_mod
        res = run_gpu(args, rank, world, local_rank, dist)
        if dist is not None:
            dist.destroy_process_group()
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
