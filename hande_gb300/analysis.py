"""Blocking analysis of FCIQMC report data.

The role of pyhande's analysis of HANDE output (tools/pyhande, which reblocks
with tools/pyblock/pyblock/blocking.py): serial correlation between reports is
removed by repeatedly averaging neighbouring data points (Flyvbjerg and
Petersen, J. Chem. Phys. 91, 461 (1989)); the standard error is read at the
smallest block length B with B^3 > 2 N (sigma_B / sigma_0)^4 (Lee, Needs et
al., Phys. Rev. E 83, 066706 (2011)), the criterion pyblock applies.  The
projected energy is the ratio of the reblocked means of sum_j H_0j N_j and N_0,
with its error from their reblocked covariance."""

from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence

import numpy as np


@dataclass
class Block:
    block: int        # blocking iteration (block length 2**block)
    ndata: int        # data points at this iteration
    mean: np.ndarray  # mean of each variable
    cov: np.ndarray   # covariance matrix of the variables
    std_err: np.ndarray
    std_err_err: np.ndarray


def reblock(data: np.ndarray) -> List[Block]:
    """data: (nvar, ndata) or (ndata,).  One entry per blocking iteration."""
    x = np.atleast_2d(np.asarray(data, dtype=float))
    out = []
    b = 0
    while x.shape[1] >= 2:
        n = x.shape[1]
        mean = x.mean(axis=1)
        cov = np.atleast_2d(np.cov(x, ddof=1))
        se = np.sqrt(np.diag(cov) / n)
        out.append(Block(b, n, mean, cov, se, se / np.sqrt(2.0 * (n - 1))))
        m = (n // 2) * 2
        x = 0.5 * (x[:, 0:m:2] + x[:, 1:m:2])
        b += 1
    return out


def optimal_block(blocks: Sequence[Block]) -> int:
    """Index of the optimal blocking iteration (largest over the variables),
    or -1 when no iteration satisfies the criterion (too little data)."""
    n0 = blocks[0].ndata
    se0 = blocks[0].std_err
    best = -1
    for v in range(len(se0)):
        opt = -1
        for blk in blocks:
            B = 2.0 ** blk.block
            if se0[v] == 0.0 or B ** 3 > 2.0 * n0 * (blk.std_err[v] / se0[v]) ** 4:
                opt = blk.block
                break
        if opt < 0:
            return -1
        best = max(best, opt)
    return best


def _ratio_error(blk: Block, e: float, mn: float, md: float) -> float:
    c = blk.cov / blk.ndata
    var = e * e * (c[0, 0] / mn ** 2 + c[1, 1] / md ** 2 - 2.0 * c[0, 1] / (mn * md))
    return float(np.sqrt(max(var, 0.0)))


def projected_energy(numerator: Sequence[float], d0: Sequence[float], min_blocks: int = 16):
    """Reblocked E_proj = <sum_j H_0j N_j> / <N_0> (the E_proj of a report is
    that ratio of its averages) and its standard error; returns
    (E_proj, error, optimal block).  Without an optimal block (too little data
    for the criterion) the error is the largest over the iterations that keep
    at least min_blocks blocks, a conservative estimate, and the block is -1."""
    blocks = reblock(np.vstack([np.asarray(numerator, float), np.asarray(d0, float)]))
    opt = optimal_block(blocks)
    mn, md = blocks[0].mean
    e = mn / md
    if opt >= 0:
        return e, _ratio_error(blocks[opt], e, mn, md), opt
    errs = [_ratio_error(b, e, mn, md) for b in blocks if b.ndata >= min_blocks]
    return e, max(errs) if errs else float("nan"), -1


def mean_error(series: Sequence[float], min_blocks: int = 16):
    """Reblocked mean and standard error of one series (e.g. the shift).
    Without an optimal block the error is the largest over the iterations that
    keep at least min_blocks blocks (conservative; the block is then -1)."""
    blocks = reblock(np.asarray(series, float))
    opt = optimal_block(blocks)
    if opt < 0:
        errs = [float(b.std_err[0]) for b in blocks if b.ndata >= min_blocks]
        return float(blocks[0].mean[0]), max(errs) if errs else float("nan"), opt
    return float(blocks[0].mean[0]), float(blocks[opt].std_err[0]), opt
