"""Batches of independent calculations (hgpu_batch_*): one graph launch per
cycle advances every handle; each handle must end exactly where it ends when
run on its own (same counter-based streams, no shared state)."""

import numpy as np
import pytest

from hande_gb300 import systems
from hande_gb300._abi import make_config
from tests.test_gpu_parity import engine

pytestmark = pytest.mark.gpu


def _members():
    hub3 = systems.hubbard_k([[3, 0], [0, 3]], 7, U=2.0, ms=1)
    hub4 = systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0)
    mol = systems.synthetic_molecule(12, 6, seed=4)
    return [
        (hub3, dict(tau=0.02, init_pop=50, target_population=2000, seed=3)),
        (hub4, dict(tau=0.005, init_pop=10, target_population=5000, seed=7, excit_gen="no_renorm")),
        (mol, dict(tau=2e-3, init_pop=300, target_population=3000, real_amplitudes=True, seed=11,
                   initiator=True)),
        (hub4, dict(tau=0.005, init_pop=20, target_population=4000, seed=8, nspaces=2)),
    ]


def _make(members):
    out = []
    for s, kw in members:
        cfg = make_config(s, ncycles=10, state_size=400000, spawned_state_size=400000, **kw)
        g = engine(s, cfg)
        g.initial_distribution()
        out.append(g)
    return out


@pytest.mark.parametrize("flip_one", [False, True])
def test_batch_matches_individual_runs(flip_one):
    from hande_gb300.engine import Batch
    members = _members()
    solo = _make(members)
    batched = _make(members)
    if flip_one:
        # an empty annihilation flips one handle's buffer parity: the batch
        # must follow mixed parities
        for g in (solo[1], batched[1]):
            g.annihilate_fixed(np.zeros((0, 1 + 1 + 1), np.int64), 1)
    batch = Batch(batched)
    for rep in range(5):
        rb = batch.run_report()
        for g, r in zip(solo, rb):
            rs = g.run_report()
            assert r.error_flags == 0 and rs.error_flags == 0
            assert list(r.nparticles) == list(rs.nparticles)
            assert list(r.shift) == list(rs.shift)
            assert r.nattempts == rs.nattempts
            assert r.nspawn_events == rs.nspawn_events
    for a, b in zip(solo, batched):
        sa, pa, ka = a.walkers()
        sb, pb, kb = b.walkers()
        np.testing.assert_array_equal(sa, sb)
        np.testing.assert_array_equal(pa, pb)
        np.testing.assert_array_equal(ka, kb)
        assert sa.shape[0] > 5
    batch.close()


def test_batch_rejects_duplicates():
    from hande_gb300.engine import Batch, HgpuError
    s = systems.hubbard_k([[3, 0], [0, 3]], 7, U=2.0, ms=1)
    g = engine(s, make_config(s, tau=0.02, state_size=1000, spawned_state_size=1000))
    with pytest.raises(HgpuError):
        Batch([g, g])


def test_launch_shape_changes_nothing_but_speed():
    """Handles of a batch with other launch shapes (spawn chunk, block counts),
    changed between reports as the autotuner does, end where the solo runs with
    the default shapes end; out-of-range shapes are refused."""
    from hande_gb300.engine import Batch, HgpuError
    members = _members()
    solo = _make(members)
    batched = _make(members)
    batch = Batch(batched)
    shapes = [(32, 1, 1, 1), (64, 7, 3, 5), (128, 300, 1024, 64), (96, 2, 17, 3)]
    for rep in range(4):
        for k, g in enumerate(batched):
            g.set_launch(*shapes[(k + rep) % len(shapes)])
        rb = batch.run_report()
        for g, r in zip(solo, rb):
            rs = g.run_report()
            assert r.error_flags == 0 and rs.error_flags == 0
            assert list(r.nparticles) == list(rs.nparticles)
            assert r.nattempts == rs.nattempts
    for a, b in zip(solo, batched):
        sa, pa, _ = a.walkers()
        sb, pb, _ = b.walkers()
        np.testing.assert_array_equal(sa, sb)
        np.testing.assert_array_equal(pa, pb)
    assert batched[2].launch().as_tuple() == shapes[(2 + 3) % len(shapes)]
    for bad in [(16, 1, 1, 1), (48, 1, 1, 1), (512, 1, 1, 1), (64, 0, 1, 1), (64, 1, 1025, 1), (64, 1, 1, 0)]:
        with pytest.raises(HgpuError):
            batched[0].set_launch(*bad)
    batch.close()


def test_autotuner_keeps_lists_and_results():
    """The tuner restores every list and state it times on: a batch tuned and
    then run ends where the untuned solo runs end."""
    from hande_gb300.autotune import BatchTuner
    from hande_gb300.engine import Batch
    members = _members()
    solo = _make(members)
    batched = _make(members)
    for g in solo + batched:
        g.run_report()
    batch = Batch(batched)
    tuner = BatchTuner(batch, batched, trial_cycles=1)
    choice, base, best = tuner.tune()
    assert best <= base and len(tuner.table) >= 16
    for rep in range(3):
        rb = batch.run_report()
        for g, r in zip(solo, rb):
            rs = g.run_report()
            assert list(r.nparticles) == list(rs.nparticles)
    for a, b in zip(solo, batched):
        np.testing.assert_array_equal(a.walkers()[0], b.walkers()[0])
        np.testing.assert_array_equal(a.walkers()[1], b.walkers()[1])
    batch.close()
