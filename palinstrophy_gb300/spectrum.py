"""Energy-spectrum samples and their simulation-time average.

Mirrors the reference's spectrum API (palinstrophy/turbo_simulator.py):
  compute_energy_spectrum_uv_bins      2360-2383 (binning on the GPU: pal_energy_spectrum)
  SpectrumSample / SpectrumAverageState 813-843
  update_spectrum_average (trapezoid in simulation time), initialise, mark since
  restart, mean energy, kind, CSV writers  2386-2622
The bookkeeping is host-side, as in the reference; only the O(N^2) binning runs
on the device.
"""
from __future__ import annotations

import csv
import io
import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class SpectrumSample:
    nbins: int = 0
    r_max: float = 0.0
    k_nyq: float = 0.0
    energy: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    count: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))


@dataclass
class SpectrumAverageState:
    initialized: bool = False
    has_previous: bool = False
    since_restart: bool = False
    Nbase: int = 0
    NX_full: int = 0
    NZ_full: int = 0
    NK_full: int = 0
    nbins: int = 0
    sample_count: int = 0
    first_step: int = 0
    last_step: int = 0
    r_max: float = 0.0
    k_nyq: float = 0.0
    total_dt: float = 0.0
    previous_time: float = 0.0
    first_time: float = 0.0
    last_time: float = 0.0
    previous_energy: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    integral_energy: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    count: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))


def _field_of(S):
    return S.field if hasattr(S, "field") else S


def compute_energy_spectrum_uv_bins(S) -> SpectrumSample:
    """nbins = max(32, 2N), r_max = sqrt 2, k_nyq = N/2 (turbo_simulator.py:2360-2383)."""
    if S is None:
        raise ValueError("DnsState is required")
    f = _field_of(S)
    n = int(f.N)
    nbins = max(32, 2 * n)
    r_max = math.sqrt(2.0)
    k_nyq = 0.5 * float(n)
    e, c = f.energy_spectrum(nbins, r_max, k_nyq)
    return SpectrumSample(nbins=nbins, r_max=r_max, k_nyq=k_nyq, energy=e, count=c)


def _geometry(S):
    f = _field_of(S)
    n = int(f.N)
    m = 3 * n // 2
    return n, m, m, m // 2 + 1


def mark_spectrum_average_since_restart(average: SpectrumAverageState, S=None) -> None:
    average.__dict__.update(SpectrumAverageState().__dict__)
    average.since_restart = True
    if S is not None:
        average.Nbase, average.NX_full, average.NZ_full, average.NK_full = _geometry(S)


def initialize_spectrum_average_from_sample(average, S, sample, sim_time, step) -> None:
    keep = bool(average.since_restart)
    average.__dict__.update(SpectrumAverageState().__dict__)
    average.initialized = True
    average.has_previous = True
    average.since_restart = keep
    average.Nbase, average.NX_full, average.NZ_full, average.NK_full = _geometry(S)
    average.nbins = int(sample.nbins)
    average.sample_count = 1
    average.first_step = average.last_step = int(step)
    average.r_max = float(sample.r_max)
    average.k_nyq = float(sample.k_nyq)
    average.previous_time = average.first_time = average.last_time = float(sim_time)
    average.previous_energy = np.asarray(sample.energy, np.float64).copy()
    average.integral_energy = np.zeros_like(average.previous_energy)
    average.count = np.asarray(sample.count, np.int32).copy()


def update_spectrum_average(average, S, sample, sim_time, step) -> bool:
    """Trapezoid rule in simulation time over successive samples."""
    if sample.nbins <= 0 or sample.energy.size == 0 or sample.energy.shape != sample.count.shape:
        return False
    if not average.initialized:
        initialize_spectrum_average_from_sample(average, S, sample, sim_time, step)
        return True
    geo = _geometry(S)
    if (geo != (average.Nbase, average.NX_full, average.NZ_full, average.NK_full)
            or average.nbins != int(sample.nbins)
            or average.previous_energy.shape != sample.energy.shape):
        return False
    e = np.asarray(sample.energy, np.float64)
    average.count = np.asarray(sample.count, np.int32).copy()
    average.r_max, average.k_nyq = float(sample.r_max), float(sample.k_nyq)
    sim_time, step = float(sim_time), int(step)
    if not average.has_previous:
        average.has_previous = True
        average.previous_energy = e.copy()
        average.previous_time = average.first_time = average.last_time = sim_time
        average.first_step = average.last_step = step
        average.sample_count = 1
        return True
    if sim_time <= average.previous_time or step == average.last_step:
        average.previous_energy = e.copy()
        average.previous_time = average.last_time = sim_time
        average.last_step = step
        if average.sample_count == 0:
            average.sample_count = 1
            average.first_time, average.first_step = sim_time, step
        return True
    dt = sim_time - average.previous_time
    average.integral_energy += 0.5 * dt * (average.previous_energy + e)
    average.total_dt += dt
    average.previous_energy = e.copy()
    average.previous_time = average.last_time = sim_time
    average.last_step = step
    average.sample_count += 1
    return True


def sample_and_update_spectrum_average(S, average, sim_time=None, step=None) -> bool:
    sample = compute_energy_spectrum_uv_bins(S)
    if sim_time is None:
        sim_time = float(getattr(S, "t", 0.0))
    if step is None:
        step = int(getattr(S, "it", 0))
    return update_spectrum_average(average, S, sample, float(sim_time), int(step))


def spectrum_average_kind(average) -> str:
    if average.total_dt > 0.0:
        return "simulation-time trapezoid since restart" if average.since_restart else "simulation-time trapezoid"
    return "single snapshot since restart" if average.since_restart else "single snapshot"


def spectrum_average_mean_energy(average) -> np.ndarray:
    if not average.initialized or not average.has_previous or average.previous_energy.size == 0:
        raise ValueError("no spectrum samples accumulated")
    if average.total_dt > 0.0:
        return average.integral_energy / average.total_dt
    return average.previous_energy.copy()


def _comment_line(values) -> str:
    buf = io.StringIO()
    csv.writer(buf, lineterminator="").writerow(values)
    return "# " + buf.getvalue() + "\n"


def save_energy_spectrum_csv_data(filename, energy, count, r_max, meta_header=None, meta_row=None,
                                  average=None, average_kind=None) -> None:
    e = np.asarray(energy, np.float64)
    c = np.asarray(count, np.int64)
    nbins = min(e.size, c.size)
    header, values = list(meta_header or ()), list(meta_row or ())
    if average is not None and average_kind is not None:
        header += ["AVERAGE_KIND", "SPECTRUM_SAMPLES", "T_START", "T_END", "TOTAL_DT", "FIRST_STEP", "LAST_STEP"]
        values += [average_kind, int(average.sample_count), float(average.first_time), float(average.last_time),
                   float(average.total_dt), int(average.first_step), int(average.last_step)]
    with open(filename, "w", newline="") as f:
        if header and values:
            f.write(_comment_line(header))
            f.write(_comment_line(values))
        w = csv.writer(f)
        w.writerow(("normalized_radius", "shell_sum_energy", "count"))
        for i in range(nbins):
            if c[i] > 0 and e[i] > 0.0:
                r0 = float(r_max) * i / nbins
                r1 = float(r_max) * (i + 1) / nbins
                w.writerow((0.5 * (r0 + r1), e[i], int(c[i])))


def save_energy_spectrum_uv_csv(S, filename, meta_header=None, meta_row=None) -> None:
    s = compute_energy_spectrum_uv_bins(S)
    save_energy_spectrum_csv_data(filename, s.energy, s.count, s.r_max, meta_header, meta_row)


def save_spectrum_average_csv(average, filename, meta_header=None, meta_row=None) -> None:
    save_energy_spectrum_csv_data(filename, spectrum_average_mean_energy(average), average.count, average.r_max,
                                  meta_header, meta_row, average, spectrum_average_kind(average))
