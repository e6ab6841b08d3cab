"""Roofline arithmetic of one FCIQMC cycle.

Algorithmic bytes (HANDE's data model, src/qmc_data.f90:644-671 and
src/spawn_data.F90:63-71, 8-byte words):
  E_m = 8W + 8R + 8          bytes per main-list entry (det, pops, K_ii)
  E_s = 8(W + R [+ 1])       bytes per spawned entry (det, pops [, flag])
  spawning       reads N E_m, writes S E_s
  annihilation   sort 2 S E_s, self-annihilation S E_s + S_u E_s,
                 merge N E_m + S_u E_s + N' E_m
with N / N' the main-list sizes before / after, S spawned and S_u unique
spawned entries."""

from __future__ import annotations

import os

# DRAM bytes (read + write) per spawning attempt of one k_spawn launch, measured
# by Nsight Compute on the 26-orbital synthetic molecule at 3.05e6 attempts
# (profiles/k_spawn_mol26.md: 18.87 MB read + 7.31 MB written); the traffic of a
# launch grows in proportion to its attempts (parents read once, spawned entries
# written once), so the bench scales it by the attempts of its own cycle.
SPAWN_DRAM_BYTES_PER_ATTEMPT = (18.87e6 + 7.31e6) / 3.0548e6

# What bounds k_spawn instead of HBM, from the same capture: issue slots and the
# integer (ALU) pipe, in percent of peak over the kernel's active cycles.
SPAWN_ISSUE_ACTIVE_PCT = 52.6
SPAWN_ALU_PIPE_PCT = 49.3
# Issue-slot utilisation of k_annihilate on the same workload
# (profiles/k_annihilate_mol26.md).
ANNIHILATE_ISSUE_ACTIVE_PCT = 45.7


def entry_bytes(W: int, R: int, initiator: bool):
    return 8 * W + 8 * R + 8, 8 * (W + R + (1 if initiator else 0))


def roofline_figures(phases: dict, counts: dict, W: int, R: int, initiator: bool, peaks: dict):
    Em, Es = entry_bytes(W, R, initiator)
    N, S, U, N2, A = counts["N"], counts["spawned"], counts["unique"], counts["N_after"], counts["attempts"]
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    if not peak:
        peak = 6800.0
    t_spawn = phases["spawn"] * 1e-3
    spawn_bytes = N * Em + S * Es
    ach = spawn_bytes / t_spawn / 1e9 if t_spawn > 0 else 0.0
    traffic = None
    if SPAWN_DRAM_BYTES_PER_ATTEMPT:
        traffic = SPAWN_DRAM_BYTES_PER_ATTEMPT * A
    roof = {"kernel": "k_spawn", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "traffic": traffic, "peak_source": peak_src,
            "algorithmic_bytes": spawn_bytes,
            "ncu_issue_active_pct": SPAWN_ISSUE_ACTIVE_PCT, "ncu_alu_pipe_pct": SPAWN_ALU_PIPE_PCT,
            "note": "spawning is bound by integer issue (Philox, bit manipulation, generator logic), not by HBM; "
                    "the ncu_* figures (profiles/k_spawn_mol26.md) give the issue and ALU-pipe utilisation"}
    t_ann = (phases["sort"] + phases["splits"] + phases["annihilate"]) * 1e-3
    ann_bytes = 3 * S * Es + 2 * U * Es + N * Em + N2 * Em
    ach2 = ann_bytes / t_ann / 1e9 if t_ann > 0 else 0.0
    annih = {"phases": ["sort", "splits", "annihilate"], "bound": "hbm", "achieved": ach2, "peak": peak,
             "unit": "GB/s", "frac": ach2 / peak, "algorithmic_bytes": ann_bytes, "seconds": t_ann,
             "peak_source": peak_src,
             "ncu_k_annihilate_issue_active_pct": ANNIHILATE_ISSUE_ACTIVE_PCT,
             "note": "the annihilation kernel moves its algorithmic bytes once (DRAM traffic 1.04x of them) and "
                     "is bound by instructions (Philox rounding and exact K_ii of new determinants, the merge "
                     "walk) and shared-memory latency; profiles/k_annihilate_mol26.md"}
    return roof, annih
