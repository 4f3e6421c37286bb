"""Generate the golden fixtures in this directory from the reference itself.

Run in a container that has the reference checked out (read-only is fine):

    python tests/golden/make_golden.py <path to the reference checkout>

It imports palinstrophy.turbo_simulator from that checkout, uses its own
generator and its own FP32 CPU (NumPy/scipy.fft) step functions, and writes
small .npz fixtures.  The fixtures are committed; nothing at test time reads
the reference checkout.

Fixtures
  init_<spec>_N<N>_s<seed>_k<K0>.npz : om2, uc_low, visc, Energy, WiWi, seed_out
  run_<method>_N<N>_s<seed>.npz       : om2/fnm1 after 1, 10, 100 steps, the
                                        (it, t, dt, cn, cflm) log of every next_dt
                                        call, and the initial cflm/dt
"""
from __future__ import annotations

import contextlib
import io
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(root):
    sys.path.insert(0, root)
    with contextlib.redirect_stdout(io.StringIO()):
        from palinstrophy import turbo_simulator as ts  # noqa: E402
    return ts


def _state(ts, N, Re, K0, cfl, seed, spec):
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        S = ts.create_dns_state(N=N, Re=Re, K0=K0, CFL=cfl, backend="cpu", seed=seed,
                                start_spectrum=spec, populate_compact_ur=False)
    out = buf.getvalue()

    def grab(label):
        for line in out.splitlines():
            if line.strip().startswith(label):
                return float(line.split("=")[1])
        raise KeyError(label)

    info = {"Energy": grab("Energy"), "WiWi": grab("WiWi"), "seed_out": grab("PAO seed out")}
    return S, info


def make_init(ts, N, K0, seed, spec, Re=1e4):
    S, info = _state(ts, N, Re, K0, 0.5, seed, spec)
    uc_low = np.array(S.uc_full[0:2, :N, :N // 2])
    path = os.path.join(HERE, f"init_{spec}_N{N}_s{seed}_k{int(K0)}.npz")
    np.savez_compressed(path, om2=np.array(S.om2), uc_low=uc_low, visc=np.float32(S.visc),
                        Energy=info["Energy"], WiWi=info["WiWi"], seed_out=int(info["seed_out"]),
                        N=N, K0=K0, seed=seed, Re=Re, spectrum=spec)
    print("wrote", path)
    return S


def make_run(ts, N, Re, K0, cfl, seed, spec, method, steps=100, update=10):
    S, _ = _state(ts, N, Re, K0, cfl, seed, spec)
    om2_0 = np.array(S.om2)
    uc_low_0 = np.array(S.uc_full[0:2, :N, :N // 2])
    import scipy.fft as spfft
    snaps = {}
    log = []
    with spfft.set_workers(1):
        ts.dns_step2a(S)
        ur0 = np.array(S.ur_full[0:2])
        cflm0 = float(ts.compute_cflm(S))
        S.dt = S.cflnum / (cflm0 * math.pi)
        S.cn, S.cnm1, S.t = 1.0, 0.0, 0.0
        dt0 = S.dt
        for it in range(1, steps + 1):
            S.it = it
            dt_old = S.dt
            if method == "LS_IMEX_RK3":
                ts.dns_step_ls_imex_rk3(S)
            else:
                ts.dns_step2b(S)
                ts.dns_step3(S)
                ts.dns_step2a(S)
            if it % update == 0 or it == 1 or it == steps:
                cflm = float(ts.next_dt(S))
                U, L, tau = S.flow_eddy_metrics()
                log.append((it, S.t, S.dt, S.cn, cflm, U, L))
            S.t += dt_old
            if it in (1, 10, steps):
                snaps[it] = (np.array(S.om2), np.array(S.fnm1))
        ur_end = np.array(S.ur_full[0:2])
    path = os.path.join(HERE, f"run_{method}_N{N}_s{seed}.npz")
    kw = {}
    for it, (o, f) in snaps.items():
        kw[f"om2_{it}"] = o
        kw[f"fnm1_{it}"] = f
    np.savez_compressed(path, om2_0=om2_0, uc_low_0=uc_low_0, visc=np.float32(S.visc),
                        log=np.array(log), cflm0=cflm0, dt0=dt0, ur0_checksum=ur0.astype(np.float64).sum(axis=(1, 2)),
                        ur0_absmax=np.abs(ur0).max(), ur0_sample=ur0[:, ::7, ::5],
                        ur_end_sample=ur_end[:, ::7, ::5], N=N, Re=Re, K0=K0, cfl=cfl,
                        seed=seed, spectrum=spec, method=method, steps=steps, update=update, **kw)
    print("wrote", path)


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    ts = _import_reference(root)
    # generator known-answer fixtures
    make_init(ts, 64, 10.0, 4895, "KM3")
    make_init(ts, 128, 15.0, 4895, "KM3")
    make_init(ts, 256, 10.0, 4895, "KM3")
    make_init(ts, 64, 12.0, 7, "PAO")
    make_init(ts, 128, 15.0, 4895, "PAO")
    # step fixtures from the reference FP32 CPU path
    make_run(ts, 64, 1e4, 10.0, 0.75, 4895, "KM3", "CNAB2")
    make_run(ts, 64, 1e4, 10.0, 0.5, 4895, "KM3", "LS_IMEX_RK3")
    make_run(ts, 128, 1e4, 15.0, 0.1, 4895, "PAO", "LS_IMEX_RK3", steps=100, update=25)
    make_run(ts, 256, 1e4, 10.0, 0.75, 4895, "KM3", "CNAB2", steps=100, update=100)


if __name__ == "__main__":
    main()
