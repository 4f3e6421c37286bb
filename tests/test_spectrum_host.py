"""Host bookkeeping of the energy-spectrum time average (no GPU needed)."""
import numpy as np

from palinstrophy_gb300 import spectrum as sp


class _FakeField:
    def __init__(self, N):
        self.N = N


class _FakeState:
    def __init__(self, N):
        self.field = _FakeField(N)


def _sample(vals):
    e = np.asarray(vals, np.float64)
    return sp.SpectrumSample(nbins=e.size, r_max=2 ** 0.5, k_nyq=32.0, energy=e, count=np.ones(e.size, np.int32))


def test_trapezoid_average_in_simulation_time():
    S = _FakeState(64)
    avg = sp.SpectrumAverageState()
    times = [0.0, 0.1, 0.3, 0.6]
    vals = [np.array([1.0, 2.0]), np.array([3.0, 2.0]), np.array([5.0, 1.0]), np.array([1.0, 1.0])]
    for i, (t, v) in enumerate(zip(times, vals)):
        assert sp.update_spectrum_average(avg, S, _sample(v), t, i)
    integ = sum(0.5 * (times[i + 1] - times[i]) * (vals[i] + vals[i + 1]) for i in range(3))
    np.testing.assert_allclose(sp.spectrum_average_mean_energy(avg), integ / 0.6)
    assert avg.sample_count == 4 and sp.spectrum_average_kind(avg) == "simulation-time trapezoid"


def test_repeated_step_replaces_previous_sample():
    S = _FakeState(64)
    avg = sp.SpectrumAverageState()
    sp.update_spectrum_average(avg, S, _sample([1.0]), 0.0, 0)
    sp.update_spectrum_average(avg, S, _sample([7.0]), 0.0, 0)
    assert avg.total_dt == 0.0
    np.testing.assert_allclose(sp.spectrum_average_mean_energy(avg), [7.0])
    assert sp.spectrum_average_kind(avg) == "single snapshot"


def test_geometry_change_is_rejected_and_restart_marks():
    avg = sp.SpectrumAverageState()
    sp.update_spectrum_average(avg, _FakeState(64), _sample([1.0, 2.0]), 0.0, 0)
    assert not sp.update_spectrum_average(avg, _FakeState(128), _sample([1.0, 2.0]), 1.0, 1)
    sp.mark_spectrum_average_since_restart(avg, _FakeState(128))
    assert avg.since_restart and not avg.initialized
    sp.update_spectrum_average(avg, _FakeState(128), _sample([1.0, 2.0]), 1.0, 1)
    assert sp.spectrum_average_kind(avg) == "single snapshot since restart"


def test_csv_writer(tmp_path):
    avg = sp.SpectrumAverageState()
    S = _FakeState(64)
    sp.update_spectrum_average(avg, S, _sample([1.0, 0.0, 2.0]), 0.0, 0)
    sp.update_spectrum_average(avg, S, _sample([3.0, 0.0, 2.0]), 0.5, 5)
    path = tmp_path / "spec.csv"
    sp.save_spectrum_average_csv(avg, str(path), ["N"], [64])
    lines = path.read_text().splitlines()
    assert lines[0].startswith("# N,AVERAGE_KIND")
    assert lines[2] == "normalized_radius,shell_sum_energy,count"
    assert len(lines) == 5  # two non-empty bins
