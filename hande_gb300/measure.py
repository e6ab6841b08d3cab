"""Roofline arithmetic of one FCIQMC cycle.

Algorithmic bytes (HANDE's data model, src/qmc_data.f90:644-671 and
src/spawn_data.F90:63-71, 8-byte words):
  E_m = 8W + 8R + 8          bytes per main-list entry (det, pops, K_ii)
  E_s = 8(W + R [+ 1])       bytes per spawned entry (det, pops [, flag])
  spawning       reads N E_m, writes S E_s
  annihilation   sort 2 S E_s, self-annihilation S E_s + S_u E_s,
                 merge N E_m + S_u E_s + N' E_m
with N / N' the main-list sizes before / after, S spawned and S_u unique
spawned entries.

Everything under "achieved", "frac", "algorithmic_bytes", "seconds" and
"sort_bytes_moved" is computed from the run's own device times and list sizes.
Figures that only a profiler measures (issue-slot and pipe utilisation, DRAM
bytes of a launch) come from the Nsight Compute captures recorded in
profiles/ncu_figures.json and are reported under "from_profile" with the
capture's workload and build."""

from __future__ import annotations

import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROFILE_FIGURES = os.path.join(ROOT, "profiles", "ncu_figures.json")


def profile_figures() -> dict:
    try:
        return json.load(open(PROFILE_FIGURES))
    except (OSError, ValueError):
        return {}


def entry_bytes(W: int, R: int, initiator: bool):
    return 8 * W + 8 * R + 8, 8 * (W + R + (1 if initiator else 0))


def roofline_figures(phases: dict, counts: dict, W: int, R: int, initiator: bool, peaks: dict):
    Em, Es = entry_bytes(W, R, initiator)
    N, S, U, N2, A = counts["N"], counts["spawned"], counts["unique"], counts["N_after"], counts["attempts"]
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    if not peak:
        peak = 6800.0
    prof = profile_figures()
    t_spawn = phases["spawn"] * 1e-3
    spawn_bytes = N * Em + S * Es
    ach = spawn_bytes / t_spawn / 1e9 if t_spawn > 0 else 0.0
    roof = {"kernel": "k_spawn", "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_source": peak_src, "algorithmic_bytes": spawn_bytes,
            "seconds": t_spawn, "traffic": None,
            "note": "spawning is bound by instruction issue (Philox, bit manipulation, generator logic), not by "
                    "HBM; from_profile gives the issue and pipe utilisation of a captured launch"}
    ps = prof.get("k_spawn")
    if ps:
        per_att = (ps["dram_bytes_read"] + ps["dram_bytes_write"]) / ps["attempts"]
        roof["traffic"] = per_att * A
        roof["traffic_source"] = ("DRAM bytes per attempt of the captured launch (%s) x this cycle's %d attempts"
                                  % (ps["workload"], A))
        roof["from_profile"] = dict(ps, source=os.path.relpath(PROFILE_FIGURES, ROOT))
    t_sort = phases["sort"] * 1e-3
    t_ann = (phases["sort"] + phases["splits"] + phases["annihilate"]) * 1e-3
    ann_bytes = 3 * S * Es + 2 * U * Es + N * Em + N2 * Em
    ach2 = ann_bytes / t_ann / 1e9 if t_ann > 0 else 0.0
    passes = counts.get("sort_passes", 0)
    sort_moved = counts.get("sort_bytes_per_entry", 0) * S  # what the passes read and write
    annih = {"phases": ["sort", "splits", "annihilate"], "bound": "hbm", "achieved": ach2, "peak": peak,
             "unit": "GB/s", "frac": ach2 / peak, "algorithmic_bytes": ann_bytes, "seconds": t_ann,
             "peak_source": peak_src,
             "sort_seconds": t_sort, "sort_passes": passes, "sort_bytes_moved": sort_moved,
             "sort_algorithmic_bytes": 2 * S * Es,
             "sort_achieved_gbs": sort_moved / t_sort / 1e9 if t_sort > 0 else 0.0,
             "note": "the one-pass annihilation kernel moves its algorithmic bytes once; sort_bytes_moved is what "
                     "the radix passes read and write (packed key-and-index records, summed over the passes, x S)"}
    pa = prof.get("k_annihilate")
    if pa:
        annih["from_profile"] = dict(pa, source=os.path.relpath(PROFILE_FIGURES, ROOT))
    return roof, annih
