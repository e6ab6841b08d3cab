"""Autotuner of the launch shape of a batch of calculations.

A batch (hgpu_batch_*) advances many handles with one CUDA graph launch per
cycle; how fast that cycle runs depends on how each handle's kernels are
split -- the number of attempts a warp of the spawning kernel claims at a time
(its walkers-per-warp granularity) and the block counts of the spawning,
streaming and radix-sort kernels (hgpu_launch).  Large calculations want big
chunks and many blocks; a batch of small ones runs faster when each leaves room
for the others.  None of this changes the results (every count, sum and random
stream of a cycle is independent of the split), so the tuner simply times
candidate shapes on the batch's own walker lists -- saved on the device before
the search and restored, with every handle's state, before each trial -- and
keeps the fastest.

Search (device time per batch cycle, CUDA events of hgpu_batch_run_cycles):
1. one family for every handle: spawn chunk c in {32, 64, 128, 256} and a
   scale s in {1/4, 1/2, 1, 2} of each handle's default block counts (the ones
   hgpu_create picked from its list capacities);
2. per size class (the handles grouped into thirds by main-list capacity), the
   class's scale refined over {s/2, 2s} and its chunk over the neighbours of c,
   the other classes held at their choice.
The radix digit width of the sort is fixed at 8 bits (the one-sweep passes rank
a tile with one ballot per digit bit), so it is not searched."""

from __future__ import annotations

CHUNKS = (32, 64, 128, 256)
SCALES = (0.25, 0.5, 1.0, 2.0)


def _shape(default, chunk, scale):
    sb, gb, ob = default[1], default[2], default[3]
    return (chunk, max(1, int(round(sb * scale))), min(1024, max(1, int(round(gb * scale)))),
            max(1, int(round(ob * scale))))


class BatchTuner:
    """Tunes the launch shapes of `engines`, advanced together by `batch`."""

    def __init__(self, batch, engines, trial_cycles=2):
        self.batch = batch
        self.engines = list(engines)
        self.trial_cycles = trial_cycles
        self.defaults = [e.launch().as_tuple() for e in self.engines]
        caps = sorted(range(len(self.engines)), key=lambda i: self.engines[i].cfg.walker_length)
        n = len(caps)
        self.classes = [caps[k * n // 3:(k + 1) * n // 3] for k in range(3) if caps[k * n // 3:(k + 1) * n // 3]]
        self.table = []

    def _save(self):
        self.states = []
        for e in self.engines:
            e.snapshot()
            self.states.append(e.get_state())

    def _restore(self):
        for e, st in zip(self.engines, self.states):
            e.snapshot(restore=True)
            e.set_state(st)

    def _apply(self, choice):
        for i, e in enumerate(self.engines):
            e.set_launch(*_shape(self.defaults[i], *choice[i]))

    def _time(self, choice, label):
        """Device ms per batch cycle of one trial from the saved lists."""
        self._apply(choice)
        self._restore()
        self.batch.run_cycles(1)  # builds the graphs of this shape
        for e in self.engines:
            e.end_report()
        self._restore()
        self.batch.run_cycles(self.trial_cycles)
        ms = self.engines[0].end_report().device_ms / self.trial_cycles
        for e in self.engines[1:]:
            e.end_report()
        self.table.append({"trial": label, "ms_per_cycle": ms})
        return ms

    def tune(self):
        """Search as described above; leaves the best shape applied and the
        walker lists and states as they were.  Returns (choice, ms per cycle
        with the default shapes, ms per cycle with the choice)."""
        self._save()
        n = len(self.engines)
        default = [(256, 1.0)] * n
        base = self._time(default, "default")
        best, best_ms = list(default), base
        for c in CHUNKS:
            for s in SCALES:
                if (c, s) == (256, 1.0):
                    continue
                ms = self._time([(c, s)] * n, "all c=%d s=%g" % (c, s))
                if ms < best_ms:
                    best, best_ms = [(c, s)] * n, ms
        for k, members in enumerate(self.classes):
            c0, s0 = best[members[0]]
            ci = CHUNKS.index(c0)
            cands = [(c0, s0 / 2), (c0, s0 * 2)]
            if ci > 0:
                cands.append((CHUNKS[ci - 1], s0))
            if ci + 1 < len(CHUNKS):
                cands.append((CHUNKS[ci + 1], s0))
            for c, s in cands:
                trial = list(best)
                for i in members:
                    trial[i] = (c, s)
                ms = self._time(trial, "class %d c=%d s=%g" % (k, c, s))
                if ms < best_ms:
                    best, best_ms = trial, ms
        self._apply(best)
        self._restore()
        for e in self.engines:
            e.end_report()
        self._restore()
        self.choice = best
        return best, base, best_ms

    def summary(self):
        per_class = []
        for k, members in enumerate(self.classes):
            c, s = self.choice[members[0]]
            caps = [self.engines[i].cfg.walker_length for i in members]
            per_class.append({"class": k, "handles": len(members), "capacity_range": [min(caps), max(caps)],
                              "spawn_chunk": c, "block_scale": s})
        return per_class
