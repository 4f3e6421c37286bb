"""Benchmark: DNS steps/s at N=4096, FP32 form vs FP64 plain, on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (the large single-field configuration): N=4096 (3/2-padded 6144^2),
KM3 start K0=15 seed 4895, Re=1e5, LS-IMEX-RK3, CFL 0.1, synthetic initial
field from the package's host generator.  One "step" is one full 3-stage
LS-IMEX-RK3 step of the field (6 kernel launches).

Printed JSON line (rank 0):
  value      FP32-form steps/s, whole job (N ranks x replicas), device-timed with
             CUDA events on the handle's stream, state resident in HBM; the
             state (0.67 GB) is larger than L2, so no flush is needed.
  fp64       the plain FP64 path on the same GPU and workload
  e2e        the same metric through the C ABI from pinned host buffers: upload
             of the initial om2 + velocity band, initial NEXTDT, K steps with the
             run_dns NEXTDT cadence (host reads CFLM/dt at each update), and the
             download of the final om2, all inside the timed region
  roofline   the dominant kernel: algorithmic bytes per launch / its average
             launch duration (events between launches on the same stream), against
             MEASURED_PEAKS.json hbm_gbs
  cpu_baseline  the FP32 CPU port of the reference path (scipy.fft, the
             reference's worker count) timed on this host for a bounded sample

--impl reference times the reference's CPU implementation of the path (its FP32
NumPy/scipy.fft step, restated operation for operation in oracle/ because the
Python reference cannot be installed on the GPU host) on the same workload from
the reference generator's field (restated in oracle/), with the reference's FFT
worker count min(8, cores), for a bounded number of steps; it imports nothing
from palinstrophy_gb300.

rel_l2_fp32_vs_oracle_100_steps: the FP64 oracle runs 100 steps from the same
start in a spawned process while the GPU legs run; the FP32 form and the FP64
plain path then replay its dt / cn sequence and are compared with it.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import platform
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_GRID = 4096
K0, SEED, RE, CFL = 15.0, 4895, 1e5, 0.1
METHOD = "LS_IMEX_RK3"
UPDATE = 100
METRIC = "DNS steps/s at N=4096: FP32 form vs FP64 plain, same GB300, ω relL2≤1e-4"
WORKLOAD = ("DNS N=4096 (3/2-padded 6144^2) KM3 K0=15 seed 4895 Re=1e5 LS-IMEX-RK3 CFL 0.1, "
            "FP32 form (FP64 dt/CFL/diagnostic scalars)")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.rows)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic(kernel, prec):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{prec}_N{N_GRID}.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith("dram_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def _limiter(kernel, prec):
    """What bounds the kernel, from its committed ncu summary (issue and FMA-pipe
    activity), when one exists."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{prec}_N{N_GRID}.md")
    issue = fma = None
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("| smsp__issue_active |"):
                    issue = line.split("|")[2].strip()
                elif line.startswith("| sm__pipe_fma_cycles_active |"):
                    fma = line.split("|")[2].strip()
    except OSError:
        return None
    if issue is None:
        return None
    return (f"instruction issue and load/store latency, not DRAM bandwidth: ncu issue active {issue}, "
            f"FP32 FMA pipe {fma} (profiles/{kernel}_{prec}_N{N_GRID}.md)")


def _fp64_counts(kernel, cand):
    """(FP64 flops, FP64 pipe instructions) per launch of the FP64 plain path's
    kernel candidate `cand` at N=4096, from the committed ncu summary: flops =
    2 DFMA + DADD + DMUL thread instructions, pipe instructions = their sum."""
    path = os.path.join(ROOT, "profiles", f"kernels_fp64_N{N_GRID}.md")
    out = {}
    try:
        with open(path) as f:
            for line in f:
                for key in ("flops", "pipe_inst"):
                    tag = f"fp64_{key}_per_launch_{kernel}[{cand}]:"
                    if line.strip().startswith(tag):
                        out[key] = float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return out.get("flops"), out.get("pipe_inst")


def _fp64_roofline(om2, uc, visc):
    """The FP64 plain path against its own ceiling: counted FP64 flops per k_row /
    k_col launch (ncu instruction counts, profiles/) over the launch times measured
    here, against the FP64 FMA throughput measured here (pal_fp64_peak); and the
    same launches' algorithmic bytes against the measured HBM bandwidth."""
    from palinstrophy_gb300 import _lib as L
    F = _field("fp64", om2, uc, visc)
    ms_row, ms_col, _ = F.profile_kernels(METHOD, 2)
    desc = F.variant()["desc"]
    F.close()
    peak, peak_ms = L.fp64_peak()
    hbm, _ = _peaks()
    n2 = float(N_GRID) * N_GRID
    out = {"bound": "fp64", "unit": "TFLOP/s", "peak": peak,
           "peak_kind": f"measured: FP64 FMA-chain microbenchmark (pal_fp64_peak, {peak_ms:.1f} ms launch)",
           "kernels": desc}
    cands = {"k_row": desc.split("row[")[1].split("]")[0], "k_col": desc.split("col[")[1].split("]")[0]}
    for name, ms, nbytes in (("k_row", ms_row, 6.0 * n2 * 8), ("k_col", ms_col, (25.0 / 3.0) * n2 * 8)):
        fl, inst = _fp64_counts(name, cands[name])
        ach = fl / (ms / 1000.0) / 1e12 if fl else None
        # the FP64 pipe takes one instruction per slot whether DFMA (2 flops) or
        # DADD / DMUL (1 flop): the pipe fraction is the FFT's real ceiling
        pipe = inst / (ms / 1000.0) / (peak * 1e12 / 2.0) if inst else None
        out[name] = {"ms": ms, "candidate": cands[name], "flops_per_launch": fl, "achieved": ach,
                     "frac": ach / peak if ach else None, "pipe_inst_per_launch": inst, "pipe_frac": pipe,
                     "hbm_GBps": nbytes / (ms / 1000.0) / 1e9, "hbm_frac": nbytes / (ms / 1000.0) / 1e9 / hbm}
    dom = "k_row" if ms_row >= ms_col else "k_col"
    out["kernel"] = dom
    out["achieved"] = out[dom]["achieved"]
    out["frac"] = out[dom]["frac"]
    out["pipe_frac"] = out[dom]["pipe_frac"]
    return out


def _init_arrays():
    from palinstrophy_gb300 import _lib as L
    return L.pao_generate(N_GRID, K0, RE, SEED, "KM3")


def _field(prec, om2, uc, visc):
    from palinstrophy_gb300.turbo_simulator import Field
    F = Field(N_GRID, prec, RE, CFL)
    F.set_state(om2, None, uc)
    F.set_scalar("visc", visc)
    F.step2a()
    c0 = F.compute_cflm()
    F.set_scalar("dt", CFL / (c0 * math.pi))
    F.set_scalar("cn", 1.0)
    F.set_scalar("cnm1", 0.0)
    return F


def _timed_steps(F, steps, warmup, sampler_index=None):
    import torch
    s = torch.cuda.ExternalStream(F.stream_ptr())
    F.step(METHOD, warmup, update=UPDATE)
    F.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(sampler_index) if sampler_index is not None else None
    if clocks:
        clocks.__enter__()
        time.sleep(0.3)
    e0.record(s)
    F.step(METHOD, steps, update=UPDATE)
    e1.record(s)
    e1.synchronize()
    if clocks:
        clocks.__exit__()
    return e0.elapsed_time(e1), (clocks.summary() if clocks else None)


def _e2e(prec, om2, uc, visc, steps):
    """Whole job through the C ABI from pinned host buffers (run_dns shape)."""
    import numpy as np
    import torch
    from palinstrophy_gb300.turbo_simulator import Field
    cdt = np.complex64 if prec == "fp32" else np.complex128
    pin_om = torch.empty(om2.size * 2, dtype=torch.float32 if prec == "fp32" else torch.float64).pin_memory()
    pin_uc = torch.empty(uc.size * 2, dtype=pin_om.dtype).pin_memory()
    pin_out = torch.empty_like(pin_om).pin_memory()
    h_om = pin_om.numpy().view(cdt).reshape(om2.shape)
    h_uc = pin_uc.numpy().view(cdt).reshape(uc.shape)
    h_out = pin_out.numpy().view(cdt).reshape(om2.shape)
    h_om[...] = om2
    h_uc[...] = uc
    # one untimed pass through the same pinned buffers: the first DMA from
    # freshly pinned pages can take 10-20 ms more, a one-off cost of the buffers
    W = Field(N_GRID, prec, RE, CFL)
    W.set_state(h_om, None, h_uc)
    W._ck(W.lib.pal_get_field(W.h, 0, h_out.ctypes.data_as(__import__("ctypes").c_void_p)))
    W.close()
    F = Field(N_GRID, prec, RE, CFL)
    F.synchronize()
    t0 = time.perf_counter()
    F.set_state(h_om, None, h_uc)
    F.set_scalar("visc", visc)
    F.step2a()
    c0 = F.compute_cflm()
    F.set_scalar("dt", CFL / (c0 * math.pi))
    F.set_scalar("cn", 1.0)
    F.set_scalar("cnm1", 0.0)
    marks = sorted({1, steps} | set(range(UPDATE, steps + 1, UPDATE)))
    done = 0
    for m in marks:
        F.step(METHOD, m - done)
        done = m
        F.next_dt(sync_host=True)  # host reads CFLM/dt as run_dns does
    F._ck(F.lib.pal_get_field(F.h, 0, h_out.ctypes.data_as(__import__("ctypes").c_void_p)))
    t1 = time.perf_counter()
    F.close()
    esz = 8 if prec == "fp32" else 16
    h2d = (om2.size + uc.size) * esz
    d2h = om2.size * esz + len(marks) * 64
    return steps / (t1 - t0), h2d / steps, d2h / steps


def _ensemble_rate(steps=1000, warmup=20):
    """Batched ensemble: 96 members (32 each at N=256, 384, 512), seeds 1-96, KM3
    K0=10, Re=1e4, CNAB2, per-member adaptive dt at CFL 0.5 (NEXTDT every step,
    fused into the row pass), FP32, replayed from a CUDA graph.  Default: one
    launch per pass for all three sizes (2 per CNAB2 step); for comparison the
    per-size launches (6 per step) of candidates re-tuned on each group's
    batched shape."""
    import torch
    from palinstrophy_gb300 import _lib as L
    from palinstrophy_gb300.turbo_simulator import Ensemble
    Ns = [256] * 32 + [384] * 32 + [512] * 32
    inits = [L.pao_generate(n, 10.0, 1e4, m + 1, "KM3") for m, n in enumerate(Ns)]
    out = {}
    for mode in ("fused", "per_size_tuned"):
        E = Ensemble(Ns, "fp32", 1e4, 0.5)
        if mode == "per_size_tuned":
            E.autotune()  # candidates timed on the batched launch shape of each size group
        for m, (om2, uc, st) in enumerate(inits):
            E.set_member(m, om2, None, uc)
            E.set_scalar(m, "visc", st["visc"])
        E.init_dt()
        s = torch.cuda.ExternalStream(E.stream_ptr())
        E.step("CNAB2", warmup, update=1, graph=True)
        E.step("CNAB2", steps, update=1, graph=True)  # capture
        E.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        E.step("CNAB2", steps, update=1, graph=True)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[mode] = {"ensemble_steps_per_s": steps / (ms / 1000.0),
                     "member_steps_per_s": len(Ns) * steps / (ms / 1000.0),
                     "launches_per_step": 2 if mode == "fused" else 6,
                     "kernels": {n: E.variant(n) for n in (256, 384, 512)},
                     "sample_member_dt": sorted(E.scalars(m)["dt"] for m in (0, 40, 95))}
        E.close()
    f = out["fused"]
    return {"members": len(Ns), "sizes": [256, 384, 512], "steps": steps, "cuda_graph": True,
            "ensemble_steps_per_s": f["ensemble_steps_per_s"], "member_steps_per_s": f["member_steps_per_s"],
            "launches_per_step": 2, "one_launch_per_pass": True, "kernels": f["kernels"],
            "sample_member_dt": f["sample_member_dt"], "per_size_tuned": out["per_size_tuned"]}


def _differentiation(directions=8):
    """Gradient of the final palinstrophy after 200 fixed-dt (2e-3) LS-IMEX-RK3 steps at
    N=512, Re=5e3, PAO K0=12 seed 7, FP32, checkpoints every 20 steps: cost of the
    backward sweep against the forward run, and central differences (eps = 1e-3
    relative) of the FP64 forward along 8 seeded Gaussian directions."""
    import numpy as np
    import torch
    from palinstrophy_gb300 import _lib as L
    from palinstrophy_gb300.turbo_simulator import Field
    N, dt, Re, nsteps, ck = 512, 2e-3, 5e3, 200, 20
    om0, _, st = L.pao_generate(N, 12.0, Re, 7, "PAO")
    visc = st["visc"]

    def field(prec):
        F = Field(N, prec, Re, 0.5)
        F.set_state(om0, None, None)
        F.set_scalar("visc", visc)
        F.set_scalar("dt", dt)
        return F

    def loss_of(om):
        om = om.astype(np.complex128)
        kx = np.arange(N // 2)[None, :]
        kz = np.fft.fftfreq(N, 1.0 / N)[:, None]
        return 0.5 * float((np.where(kx == 0, 1.0, 2.0) * (kx * kx + kz * kz) * np.abs(om) ** 2).sum())

    F = field("fp32")
    s = torch.cuda.ExternalStream(F.stream_ptr())
    F.step("LS_IMEX_RK3", 5, update=0)
    F.close()
    F = field("fp32")
    F.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s = torch.cuda.ExternalStream(F.stream_ptr())
    e0.record(s)
    F.step("LS_IMEX_RK3", nsteps, update=0)
    e1.record(s)
    e1.synchronize()
    t_fwd = e0.elapsed_time(e1) / 1000.0
    F.close()
    F = field("fp32")
    F.adjoint_palinstrophy(nsteps, ck)  # warm-up: graph capture, allocator
    F.close()
    F = field("fp32")
    F.synchronize()
    t0 = time.perf_counter()
    loss, grad = F.adjoint_palinstrophy(nsteps, ck)
    t_grad = time.perf_counter() - t0
    F.close()
    F = field("fp64")
    _, grad64 = F.adjoint_palinstrophy(nsteps, ck)
    F.close()
    grad64 = grad64.astype(np.complex128)
    rng = np.random.default_rng(12345)
    errs, errs64, fds, ads, ads64 = [], [], [], [], []
    for _ in range(directions):
        d = (rng.standard_normal(om0.shape) + 1j * rng.standard_normal(om0.shape)).astype(np.complex128)
        eps = 1e-3 * np.linalg.norm(om0) / np.linalg.norm(d)
        vals = []
        for sgn in (1.0, -1.0):
            G = Field(N, "fp64", Re, 0.5)
            G.set_state(om0.astype(np.complex128) + sgn * eps * d, None, None)
            G.set_scalar("visc", visc)
            G.set_scalar("dt", dt)
            G.step("LS_IMEX_RK3", nsteps, update=0)
            vals.append(loss_of(G.om2()))
            G.close()
        fd = (vals[0] - vals[1]) / (2 * eps)
        ad = float(np.real(np.vdot(grad.astype(np.complex128), d)))
        ad64 = float(np.real(np.vdot(grad64, d)))
        errs.append(abs(fd - ad) / abs(fd))
        errs64.append(abs(fd - ad64) / abs(fd))
        fds.append(fd)
        ads.append(ad)
        ads64.append(ad64)
    return {"N": N, "steps": nsteps, "checkpoint_every": ck, "precision": "fp32", "loss": loss,
            "forward_s": t_fwd, "gradient_call_s": t_grad,
            "backward_over_forward": (t_grad - t_fwd) / t_fwd,
            "fd_directions": directions, "fd_eps_rel": 1e-3, "fd_forward": "fp64",
            "fd_max_rel_err_fp32_adjoint": max(errs), "fd_max_rel_err_fp64_adjoint": max(errs64),
            # the 8 directional derivatives as one vector: |ad - fd| / |fd|
            "fd_rel_l2_fp32_adjoint": float(np.linalg.norm(np.subtract(ads, fds)) / np.linalg.norm(fds)),
            "fd_rel_l2_fp64_adjoint": float(np.linalg.norm(np.subtract(ads64, fds)) / np.linalg.norm(fds)),
            "grad_rel_l2_fp32_vs_fp64_adjoint": float(np.linalg.norm(grad - grad64) / np.linalg.norm(grad64))}


def _rel_l2(a, b):
    import numpy as np
    a = a.astype(np.complex128)
    b = b.astype(np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _precision_form(steps=2000, update=100):
    """N=1024, labelled k^4 exp(-2 (k/15)^2) unit-energy start (seed 4895), Re=1e4,
    LS-IMEX-RK3 at CFL 0.1: the FP32 form and the FP64 plain path from the identical
    start, each with its own adaptive dt; steps/s of each and their agreement."""
    import numpy as np
    import torch
    from palinstrophy_gb300.initial import k4_unit_energy
    from palinstrophy_gb300.turbo_simulator import Field
    N, Re, cfl = 1024, 1e4, 0.1
    om2, uc = k4_unit_energy(N, 15.0, SEED)
    visc = float(np.float32(1.0 / float(np.float32(Re))))
    out = {"N": N, "start": "k4_unit_energy(K0=15, seed 4895), labelled (not the reference generator)",
           "method": METHOD, "cfl": cfl, "steps": steps, "update": update}
    res = {}
    for prec in ("fp32", "fp64"):
        F = Field(N, prec, Re, cfl)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", visc)
        F.step2a()
        F.set_scalar("dt", cfl / (F.compute_cflm() * math.pi))
        s = torch.cuda.ExternalStream(F.stream_ptr())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        F.synchronize()
        e0.record(s)
        F.step(METHOD, steps, update=update, final_update=True)
        e1.record(s)
        e1.synchronize()
        d = F.diagnostics()
        res[prec] = (F.om2(), d)
        out[prec] = {"steps_per_s": steps / (e0.elapsed_time(e1) / 1000.0), "E": d["E"], "Z": d["Z"],
                     "t": F.scalars()["t"]}
        F.close()
    out["rel_l2_om_fp32_vs_fp64"] = _rel_l2(res["fp32"][0], res["fp64"][0])
    out["rel_E_fp32_vs_fp64"] = abs(res["fp32"][1]["E"] / res["fp64"][1]["E"] - 1.0)
    out["rel_Z_fp32_vs_fp64"] = abs(res["fp32"][1]["Z"] / res["fp64"][1]["Z"] - 1.0)
    return out


def _embed_spectrum(om2, N):
    """A compact (n, n/2) rfft2 band (kz in fftfreq order, kx < n/2, amplitudes
    as irfft2(norm="forward") reads them) placed in the (N, N/2) band of a
    larger grid: the same field.  The kz = -n/2 row, which the n-grid step
    keeps at zero, is left at zero."""
    import numpy as np
    n = om2.shape[0]
    h = n // 2
    out = np.zeros((N, N // 2), dtype=om2.dtype)
    out[:h, :h] = om2[:h, :]
    out[N - h + 1:, :h] = om2[h + 1:, :]
    return out


def _large_single_field(om2, uc, visc, steps_8192=30, drift_steps=500, every=100):
    """N=8192 FP32 (KM3 K0=15 seed 4895, Re=1e5, LS-IMEX-RK3, CFL 0.1): steps/s and
    per-kernel rates; the energy / enstrophy history of the N=4096 FP32 form
    against the FP64 plain run over 500 steps from the identical start; and
    500 N=8192 FP32 steps of the same flow against that FP64 run."""
    import numpy as np
    import torch
    from palinstrophy_gb300 import _lib as L
    from palinstrophy_gb300.turbo_simulator import Field
    N = 8192
    o8, u8, st8 = L.pao_generate(N, K0, RE, SEED, "KM3")
    F = Field(N, "fp32", RE, CFL)
    F.set_state(o8, None, u8)
    F.set_scalar("visc", st8["visc"])
    F.step2a()
    F.set_scalar("dt", CFL / (F.compute_cflm() * math.pi))
    ms_row, ms_col, _ = F.profile_kernels(METHOD, 3)
    F.step(METHOD, 3, update=UPDATE)
    s = torch.cuda.ExternalStream(F.stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    F.synchronize()
    e0.record(s)
    F.step(METHOD, steps_8192, update=UPDATE)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps_8192
    variant = F.variant()["desc"]
    F.close()
    n2, s_bytes = float(N) * N, 4
    big = {"N": N, "dtype": "f32", "steps": steps_8192, "steps_per_s": 1000.0 / ms, "ms_per_step": ms,
           "kernels": variant,
           "k_row": {"ms": ms_row, "algorithmic_GBps": 6.0 * n2 * s_bytes / (ms_row / 1000.0) / 1e9},
           "k_col": {"ms": ms_col, "algorithmic_GBps": (25.0 / 3.0) * n2 * s_bytes / (ms_col / 1000.0) / 1e9}}
    # N=4096 histories, sampled every `fine` steps (NEXTDT follows the global
    # iteration count, so the sampling does not change the trajectory)
    fine = 10
    hist = {}
    for prec in ("fp32", "fp64"):
        G = _field(prec, om2, uc, visc)
        h = []
        for _ in range(drift_steps // fine):
            G.step(METHOD, fine, update=UPDATE, final_update=False)
            d = G.diagnostics()
            h.append((G.scalars()["t"], d["E"], d["Z"]))
        hist[prec] = h
        G.close()
    coarse = {p: hist[p][every // fine - 1::every // fine] for p in hist}
    dE = max(abs(a[1] / b[1] - 1.0) for a, b in zip(coarse["fp32"], coarse["fp64"]))
    dZ = max(abs(a[2] / b[2] - 1.0) for a, b in zip(coarse["fp32"], coarse["fp64"]))
    drift = {"N": N_GRID, "steps": drift_steps, "every": every,
             "E_fp64": [h[1] for h in coarse["fp64"]], "Z_fp64": [h[2] for h in coarse["fp64"]],
             "max_rel_dE_fp32_vs_fp64": dE, "max_rel_dZ_fp32_vs_fp64": dZ}
    # N=8192 FP32 from the same flow: the N=4096 start embedded in the larger
    # spectral grid (coefficients are grid-independent: irfft2 norm="forward";
    # the kz = -N/2 row, which the N=4096 step keeps at zero, stays zero), 500
    # steps; E and Z against the N=4096 FP64 run at the same physical times
    # (linear interpolation between its samples, dt being half as large here)
    big_om2 = _embed_spectrum(om2, N)
    H = Field(N, "fp32", RE, CFL)
    H.set_state(big_om2, None, None)
    H.set_scalar("visc", visc)
    H.step2a()
    H.set_scalar("dt", CFL / (H.compute_cflm() * math.pi))
    H.set_scalar("cn", 1.0)
    H.set_scalar("cnm1", 0.0)
    d0 = H.diagnostics()
    h8 = []
    for _ in range(drift_steps // every):
        H.step(METHOD, every, update=UPDATE, final_update=True)
        d = H.diagnostics()
        h8.append((H.scalars()["t"], d["E"], d["Z"]))
    H.close()
    t64 = np.array([0.0] + [h[0] for h in hist["fp64"]])
    E64 = np.array([np.nan] + [h[1] for h in hist["fp64"]])
    Z64 = np.array([np.nan] + [h[2] for h in hist["fp64"]])
    G = _field("fp64", om2, uc, visc)
    d64 = G.diagnostics()
    G.close()
    E64[0], Z64[0] = d64["E"], d64["Z"]
    cross = {"N": N, "dtype": "f32", "steps": drift_steps, "every": every,
             "start": "the N=4096 KM3 start (K0=15, seed 4895) embedded in the N=8192 spectral grid",
             "t": [h[0] for h in h8], "E": [h[1] for h in h8], "Z": [h[2] for h in h8],
             "drift_E": h8[-1][1] / d0["E"] - 1.0, "drift_Z": h8[-1][2] / d0["Z"] - 1.0,
             "fp64_N4096_drift_E_same_t": float(np.interp(h8[-1][0], t64, E64)) / d64["E"] - 1.0,
             "fp64_N4096_drift_Z_same_t": float(np.interp(h8[-1][0], t64, Z64)) / d64["Z"] - 1.0,
             "max_rel_dE_vs_fp64_N4096": max(abs(h[1] / float(np.interp(h[0], t64, E64)) - 1.0) for h in h8),
             "max_rel_dZ_vs_fp64_N4096": max(abs(h[2] / float(np.interp(h[0], t64, Z64)) - 1.0) for h in h8),
             "rel_E0_vs_N4096": d0["E"] / d64["E"] - 1.0, "rel_Z0_vs_N4096": d0["Z"] / d64["Z"] - 1.0}
    return {"N8192_fp32": big, "N4096_fp32_vs_fp64_history": drift, "N8192_fp32_vs_N4096_fp64_history": cross}


def _generator_times(N=N_GRID):
    """Initial KM3 field at N: the device generator (pal_generate) against the
    host restatement (pal_pao_generate), wall seconds after one warm-up call."""
    from palinstrophy_gb300 import _lib as L
    from palinstrophy_gb300.turbo_simulator import Field
    F = Field(N, "fp32", RE, CFL)
    F.generate(K0, RE, SEED, "KM3")
    t0 = time.perf_counter()
    F.generate(K0, RE, SEED, "KM3")
    t_dev = time.perf_counter() - t0
    F.close()
    t0 = time.perf_counter()
    L.pao_generate(N, K0, RE, SEED, "KM3")
    t_host = time.perf_counter() - t0
    return {"N": N, "spectrum": "KM3", "device_s": t_dev, "host_s": t_host}


def _cpu_port_rate(steps_cap, seconds, workers, om2, uc, visc, warmup=1):
    """FP32 CPU port of the reference path (the oracle's FP32 mode, which is the
    reference's NumPy/scipy.fft step operation for operation, with the reference's
    elementwise passes on one thread as NumPy runs them): steps/s over a bounded
    sample after `warmup` untimed steps."""
    import numpy as np
    from oracle import dns_oracle as do
    S = do.OracleState(N_GRID, om2, uc, visc, CFL, dtype=np.float32, workers=workers, threads=1)
    do.init_dt(S)
    for _ in range(warmup):
        do.rk3(S)
    n, t0 = 0, time.perf_counter()
    while n < steps_cap and (time.perf_counter() - t0) < seconds:
        do.rk3(S)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, n, dt


def _oracle_worker(N, om2, uc, visc, steps, out_dir):
    """FP64 oracle run from the identical start (spawned process, no CUDA): the
    final om2 and the NEXTDT log (it, t, dt, cn, cflm) into out_dir."""
    import numpy as np
    from oracle import dns_oracle as do
    n = os.cpu_count() or 1
    S = do.OracleState(N, om2, uc, visc, CFL, dtype=np.float64, workers=n, threads=n)
    do.init_dt(S)
    dt0 = S.dt
    log = []
    t0 = time.perf_counter()
    do.run(S, steps, METHOD, UPDATE, log=log)
    secs = time.perf_counter() - t0
    np.save(os.path.join(out_dir, "om2.npy"), S.om2)
    np.save(os.path.join(out_dir, "log.npy"), np.array([(dt0, 0, 0, 0, 0)] + log, dtype=np.float64))
    with open(os.path.join(out_dir, "secs"), "w") as f:
        f.write(f"{secs} {n}")


class _OracleRun:
    """The FP64 oracle (oracle/dns_oracle.py) for `steps` LS-IMEX-RK3 steps at
    N=4096, in a spawned process while the GPU legs run."""

    def __init__(self, om2, uc, visc, steps=100):
        import multiprocessing as mp
        import tempfile
        self.steps = steps
        self.dir = tempfile.mkdtemp(prefix="pal_oracle_")
        self.proc = mp.get_context("spawn").Process(target=_oracle_worker,
                                                    args=(om2.shape[0], om2, uc, visc, steps, self.dir))
        self.proc.start()

    def result(self, timeout=1800):
        import numpy as np
        self.proc.join(timeout)
        if self.proc.exitcode != 0:
            raise RuntimeError(f"oracle process failed (exit code {self.proc.exitcode})")
        om2 = np.load(os.path.join(self.dir, "om2.npy"))
        log = np.load(os.path.join(self.dir, "log.npy"))
        with open(os.path.join(self.dir, "secs")) as f:
            secs, threads = f.read().split()
        for name in ("om2.npy", "log.npy", "secs"):
            os.remove(os.path.join(self.dir, name))
        os.rmdir(self.dir)
        return om2, log, float(secs), int(threads)


def _vs_oracle(om2, uc, visc, oracle):
    """rel-L2 of om2 after the oracle's steps, FP32 form and FP64 plain path from
    the identical start, the oracle's dt / cn sequence replayed into the GPU run."""
    from palinstrophy_gb300.turbo_simulator import Field
    o_om2, log, secs, threads = oracle.result()
    dt0, marks = float(log[0, 0]), log[1:]
    out = {}
    for prec in ("fp32", "fp64"):
        F = Field(N_GRID, prec, RE, CFL)
        F.set_state(om2, None, uc)
        F.set_scalar("visc", visc)
        F.step2a()
        F.set_scalar("dt", dt0)
        F.set_scalar("cn", 1.0)
        F.set_scalar("cnm1", 0.0)
        done = 0
        for row in marks:
            F.step(METHOD, int(row[0]) - done, update=0)
            done = int(row[0])
            F.set_scalar("dt", float(row[2]))
            F.set_scalar("cn", float(row[3]))
        out[prec] = _rel_l2(F.om2(), o_om2)
        F.close()
    return out["fp32"], out["fp64"], {"steps": oracle.steps, "oracle_s": secs, "oracle_threads": threads,
                                      "dt_replayed": True, "oracle": "oracle/dns_oracle.py FP64 (numpy/scipy.fft)"}


def _cpu_name():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def run_reference(args):
    """The reference's CPU implementation of the path on this host: the oracle's
    FP32 port of the NumPy/scipy.fft step (pinned bit for bit to the reference's
    own outputs by tests/test_oracle_golden.py; the Python reference itself is not
    installed here), from the reference generator's N=4096 field restated in
    oracle/pao_generator.py, with the reference's FFT worker count min(8, cores).
    Nothing from palinstrophy_gb300 is imported on this path."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import pao_generator as pg
    g = pg.generate_fast(N_GRID, K0, RE, SEED, "KM3")
    workers = min(8, os.cpu_count() or 1)
    warmup = max(3, getattr(args, "warmup", 3))
    rate, n, secs = _cpu_port_rate(max(1, args.steps), 120.0, workers, g["om2"], g["uc_low"], float(g["visc"]),
                                   warmup=warmup)
    sample = (f"{n} LS-IMEX-RK3 steps at N=4096 after {warmup} warm-up steps ({secs:.1f} s), FP32 numpy/scipy.fft "
              f"port of the reference path (oracle/dns_oracle.py), scipy.fft workers={workers} "
              f"(the reference's min(8, cores)), {os.cpu_count()} host cores, {_cpu_name()}")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": n, "warmup": warmup, "ms_per_step": 1000.0 / rate, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (reference KM3 generator restated, seed 4895)",
        "config": {"workload": WORKLOAD.replace("FP32 form (FP64 dt/CFL/diagnostic scalars)",
                                                "reference FP32 CPU path (numpy + scipy.fft)"), "N": N_GRID},
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": workers, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import numpy as np
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    om2, uc, st = _init_arrays()
    visc = st["visc"]

    # FP32 form: headline
    F = _field("fp32", om2, uc, visc)
    ms_row, ms_col, _ = F.profile_kernels(METHOD, 3)
    kernels32 = F.variant()["desc"]
    F.close()
    F = _field("fp32", om2, uc, visc)
    ms32, clocks = _timed_steps(F, args.steps, args.warmup, sampler_index=local)
    F.close()
    # FP64 plain path
    k64 = max(3, args.steps // 40)
    F = _field("fp64", om2, uc, visc)
    ms64, _ = _timed_steps(F, k64, max(3, args.warmup // 10))
    F.close()

    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms32, ms64], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms32, ms64 = float(t[0]), float(t[1])
    if rank != 0:
        return

    # accuracy: FP32 form vs FP64 plain after 100 steps from the identical start
    A = _field("fp32", om2, uc, visc)
    B = _field("fp64", om2, uc, visc)
    A.step(METHOD, 100, update=UPDATE, final_update=True)
    B.step(METHOD, 100, update=UPDATE, final_update=True)
    rel = _rel_l2(A.om2(), B.om2())
    A.close()
    B.close()

    e2e_rate, h2d, d2h = _e2e("fp32", om2, uc, visc, args.steps)
    oracle = _OracleRun(om2, uc, visc, 100)
    fp64_roof = _fp64_roofline(om2, uc, visc)
    ens = _ensemble_rate()
    diff = _differentiation()
    prec_form = _precision_form()
    large = _large_single_field(om2, uc, visc)
    gen_times = _generator_times()

    rate32 = ws * args.steps / (ms32 / 1000.0)
    rate64 = ws * k64 / (ms64 / 1000.0)
    peak, peak_kind = _peaks()
    s_bytes = 4
    n2 = float(N_GRID) * N_GRID
    bytes_row = 6.0 * n2 * s_bytes   # read + write 2 planes of (N/2 x 3N/2) complex
    # the same planes + the om / fnm1 traffic of an LS-IMEX-RK3 step's three
    # column passes, in arrays of N x N/2 complex (1.0 n2 s_bytes each way):
    # om in + q out, q in + q out, q in + om and fnm1 out -> (8 + 8 + 9) / 3
    bytes_col = (25.0 / 3.0) * n2 * s_bytes
    dominant = "k_col" if ms_col >= ms_row else "k_row"
    dom_ms = max(ms_col, ms_row)
    dom_bytes = bytes_col if dominant == "k_col" else bytes_row
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    rel_oracle32, rel_oracle64, oracle_info = _vs_oracle(om2, uc, visc, oracle)
    cpu_workers = min(8, os.cpu_count() or 1)
    cpu_rate, cpu_n, cpu_s = _cpu_port_rate(20, 90.0, cpu_workers, om2, uc, visc)
    line = {
        "metric": METRIC,
        "value": rate32,
        "unit": "steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms32 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (KM3 generator, seed 4895)",
        "config": {"workload": WORKLOAD, "N": N_GRID, "M": 3 * N_GRID // 2, "method": METHOD,
                   "update": UPDATE, "l2": "state (0.67 GB FP32) larger than L2, no flush",
                   "parallelism": f"replicas x{ws}"},
        # the large nested blocks first, so that the headline keys close the line
        "ensemble": ens,
        "differentiation": diff,
        "precision_form": prec_form,
        "large_single_field": large,
        "initial_condition": gen_times,
        "oracle_check": oracle_info,
        "e2e": {"value": e2e_rate, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        # timed region = one pal_step call: 6 launches per RK3 step, the two om/fnm1
        # order conversions, and a k_phys launch if the last step ends on the NEXTDT cadence
        "gpu_launches": 6 * args.steps + 2 + int((args.warmup + args.steps) % UPDATE == 0),
        "roofline": {"bound": "hbm", "kernel": dominant, "kernels": kernels32, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": _traffic(dominant, "fp32"), "algorithmic_bytes": dom_bytes,
                     "ms_per_launch": {"k_row": ms_row, "k_col": ms_col},
                     "limiter": _limiter(dominant, "fp32"),
                     "stage_bytes_per_s": (bytes_row + bytes_col) / ((ms_row + ms_col) / 1000.0) / 1e9},
        "cpu_baseline": {"value": cpu_rate, "unit": "steps/s", "cores": cpu_workers,
                         "kind": "port",
                         "sample": f"{cpu_n} LS-IMEX-RK3 steps at N=4096 after 1 warm-up ({cpu_s:.1f} s), FP32 "
                                   f"numpy/scipy.fft port of the reference path, scipy.fft workers={cpu_workers} "
                                   f"(the reference's min(8, cores)), {_cpu_name()}"},
        "clocks": clocks,
        "fp64_roofline": fp64_roof,
        "fp64": {"value": rate64, "unit": "steps/s", "steps": k64, "ms_per_step": ms64 / k64},
        "fp32_over_fp64": rate32 / rate64,
        "rel_l2_fp32_vs_fp64_100_steps": rel,
        "rel_l2_fp64_vs_oracle_100_steps": rel_oracle64,
        "rel_l2_fp32_vs_oracle_100_steps": rel_oracle32,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ncu-case", choices=["fp32", "fp64", "ensemble"], default=None,
                    help="profiling target: init + 2 warm-up + 2 timed steps of one precision (or of the "
                         "96-member ensemble, eager launches), no JSON")
    ap.add_argument("--ncu-n", type=int, default=N_GRID,
                    help="grid size of --ncu-case (4096 or 8192 FP32 / 4096 FP64), device generator start")
    ap.add_argument("--variant", default=None,
                    help="row,col kernel candidates for --ncu-case (skips the autotuning launches)")
    args = ap.parse_args()
    if args.ncu_case == "ensemble":
        from palinstrophy_gb300 import _lib as L
        from palinstrophy_gb300.turbo_simulator import Ensemble
        Ns = [256] * 32 + [384] * 32 + [512] * 32
        E = Ensemble(Ns, "fp32", 1e4, 0.5)
        for m, n in enumerate(Ns):
            om2, uc, st = L.pao_generate(n, 10.0, 1e4, m + 1, "KM3")
            E.set_member(m, om2, None, uc)
            E.set_scalar(m, "visc", st["visc"])
        E.init_dt()
        E.step("CNAB2", 2, update=1, graph=False)
        E.step("CNAB2", 2, update=1, graph=False)
        E.synchronize()
        E.close()
        return
    if args.ncu_case:
        if args.variant:
            os.environ["PAL_AUTOTUNE"] = "0"
        if args.ncu_n != N_GRID:
            from palinstrophy_gb300.turbo_simulator import Field
            F = Field(args.ncu_n, args.ncu_case, RE, CFL)
            _, st = F.generate(K0, RE, SEED, "KM3")
            F.set_scalar("visc", st["visc"])
            F.step2a()
            F.set_scalar("dt", CFL / (F.compute_cflm() * math.pi))
        else:
            om2, uc, st = _init_arrays()
            F = _field(args.ncu_case, om2, uc, st["visc"])
        if args.variant:
            r, c = (int(x) for x in args.variant.split(","))
            F.set_variant(r, c)
        F.step(METHOD, 2)
        F.step(METHOD, 2)
        F.synchronize()
        F.close()
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
