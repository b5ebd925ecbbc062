"""One stream split across ranks (one process per GPU).

Particles are independent once the progenitor's track is known, and every
rank recomputes that track (two FP64 orbits and the release, a few ms).  A
stream is therefore split into contiguous particle ranges, one per rank,
balanced by work: particle p of a release-major stream integrates
n_steps - (p // ppr) * spr steps, so equal particle counts would give the
first rank most of the work.  Each rank integrates its range with the
sub-range form of the stream kernels (ss_stream_cfg.first_particle); the
only collective is the optional gather of the final states at the end.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np
import torch


def stream_work(p: np.ndarray, ppr: int, spr: int, n_steps: int) -> np.ndarray:
    """Particle-steps of particles [0, p) of a release-major stream."""
    p = np.asarray(p, dtype=np.int64)
    R = p // ppr
    return p * n_steps - spr * (ppr * (R * (R - 1) // 2) + (p - R * ppr) * R)


def balanced_ranges(n_particles: int, ppr: int, spr: int, n_steps: int, world: int,
                    align: int = 0) -> List[Tuple[int, int]]:
    """Contiguous ranges [p0, p1), one per rank, of about equal work, with
    boundaries on multiples of `align` (default: whole releases, ppr)."""
    align = int(align or ppr)
    N = int(n_particles)
    total = int(stream_work(N, ppr, spr, n_steps))
    cuts = [0]
    for k in range(1, world):
        target = total * k / world
        lo, hi = cuts[-1], N
        while lo < hi:  # smallest boundary whose work reaches the target
            mid = (lo + hi) // 2
            if stream_work(mid, ppr, spr, n_steps) >= target:
                hi = mid
            else:
                lo = mid + 1
        b = min(N, max(cuts[-1], int(round(lo / align)) * align))
        cuts.append(b)
    cuts.append(N)
    return [(cuts[k], cuts[k + 1]) for k in range(world)]


def gather_ranges(local: torch.Tensor, ranges: List[Tuple[int, int]], group=None) -> torch.Tensor:
    """All ranks' range results [p1 - p0, ...] assembled in particle order on
    every rank (all_gather of equal-size padded blocks; gloo or NCCL)."""
    import torch.distributed as dist
    width = max(p1 - p0 for p0, p1 in ranges)
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[:local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in ranges]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([parts[k][:p1 - p0] for k, (p0, p1) in enumerate(ranges)], dim=0)


def gen_stream_sharded(pot_base, ts, prog_w0, Msat, rank: int, world: int, *, gather: bool = True, group=None,
                       **kw):
    """gen_stream on `world` ranks: this rank integrates its balanced range
    of releases; with gather, every rank returns the whole (lead, trail),
    else (lead, trail) of its own releases and the release range."""
    from .main import _n_draw
    from .streamhelpers import gen_stream
    n_rel = len(np.asarray(ts).reshape(-1)) - 1
    ppr = 2 * _n_draw(kw.get("n_particles_per_release", 2))
    spr_hint = 1  # the balance only needs the release order, not the step size
    rel_ranges = [(p0 // ppr, p1 // ppr) for p0, p1 in
                  balanced_ranges(n_rel * ppr, ppr, spr_hint, n_rel, world)]
    r0, r1 = rel_ranges[rank]
    lead, trail = gen_stream(pot_base, ts, prog_w0, Msat, release_range=(r0, r1), **kw)[:2]
    if not gather:
        return lead, trail, (r0, r1)
    both = torch.stack([lead, trail], dim=1).contiguous()  # [n_local, 2, ...]
    full = gather_ranges(both, rel_ranges, group)
    return full[:, 0], full[:, 1]


__all__ = ["stream_work", "balanced_ranges", "gather_ranges", "gen_stream_sharded"]
