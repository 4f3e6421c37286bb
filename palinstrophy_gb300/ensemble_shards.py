"""Ensemble members shared out over processes (one GPU each) by member index.

Members are independent fields (no exchange on the data path), so rank r of W
takes a contiguous block of members from ``member_range`` and steps it as one
GB300 ensemble (``turbo_simulator.Ensemble``: one launch per pass and member
size, CUDA-graph replay).  The only communication is the host-side gather of
per-member results for reporting (``gather_rows``), through torch.distributed
object collectives on whatever process group the caller initialised.  There
is no collective on the device.
"""
from __future__ import annotations

from typing import Sequence


def member_range(n_members: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of the members owned by `rank`: contiguous, disjoint, covering
    0..n_members-1, sizes differing by at most one (the first n % world ranks
    take one more)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if n_members < 0:
        raise ValueError("negative member count")
    base, extra = divmod(n_members, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_members(members: Sequence, rank: int, world: int) -> list:
    lo, hi = member_range(len(members), rank, world)
    return list(members[lo:hi])


def gather_rows(rows: list, group=None) -> list | None:
    """Concatenate every rank's rows on rank 0, in rank order (= member order for
    `member_range` shards); other ranks get None.  Without an initialised
    process group the rows are returned as they are."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return list(rows)
    world = dist.get_world_size(group)
    parts = [None] * world if dist.get_rank(group) == 0 else None
    dist.gather_object(list(rows), parts, dst=0, group=group)
    if parts is None:
        return None
    out = []
    for p in parts:
        out.extend(p)
    return out


def run_ensemble_shard(Ns: Sequence[int], seeds: Sequence[int], rank: int, world: int, method: str = "CNAB2",
                       nsteps: int = 100, update: int = 1, K0: float = 10.0, Re: float = 1e4, cfl: float = 0.5,
                       spectrum: str = "KM3", precision: str = "fp32", return_fields: bool = False) -> list[dict]:
    """Step this rank's members (generator start per member seed, per-member
    adaptive dt) and return one row per member: index, N, seed, t, dt, cn, CFLM,
    it (and om2 with `return_fields`)."""
    from . import _lib as L
    from .turbo_simulator import Ensemble
    if len(Ns) != len(seeds):
        raise ValueError("one seed per member")
    lo, hi = member_range(len(Ns), rank, world)
    if hi == lo:
        return []
    ens = Ensemble(Ns[lo:hi], precision=precision, Re=Re, cfl=cfl)
    try:
        for m in range(hi - lo):
            om2, uc, st = L.pao_generate(int(Ns[lo + m]), K0, Re, int(seeds[lo + m]), spectrum)
            ens.set_member(m, om2, None, uc)
            ens.set_scalar(m, "visc", st["visc"])
        ens.init_dt()
        ens.step(method, nsteps, update=update, graph=True)
        ens.synchronize()
        rows = []
        for m in range(hi - lo):
            row = {"member": lo + m, "N": int(Ns[lo + m]), "seed": int(seeds[lo + m]), **ens.scalars(m)}
            if return_fields:
                row["om2"] = ens.om2(m)
            rows.append(row)
        return rows
    finally:
        ens.close()
