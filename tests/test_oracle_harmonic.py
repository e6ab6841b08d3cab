"""Harmonic population control (Yang, Pahl and Brand's shift update, the
shift_harmonic_forcing term of update_shift, src/energy_evaluation.F90:659-711)
on the oracle: with critical damping (zeta = shift_damping^2 / 4, what
shift_harmonic_crit_damp sets, src/qmc.F90:204-205) and the shift varying from
the first report, the population settles at the target; the option mapping of
the driver follows init_qmc."""

import numpy as np

from hande_gb300 import calc, systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle


def _hubbard():
    return systems.hubbard_k([[4, 0], [0, 4]], 10, U=1.0)


def _cfg(s, zeta, target):
    return make_config(s, tau=0.01, ncycles=10, seed=11, init_pop=1000, target_population=target,
                       shift_damping=0.04, shift_harmonic_forcing=zeta, vary_shift_from_proje=True,
                       state_size=400000, spawned_state_size=400000)


def test_population_settles_at_target():
    s = _hubbard()
    # an equilibrated calculation of about 3000 walkers, its shift varying
    g = Oracle(s, _cfg(s, 0.0, 3000.0))
    g.initial_distribution()
    for _ in range(400):
        r = g.run_report()
        assert r.error_flags == 0
    assert r.vary_shift[0] == 1
    walkers, state = g.walkers(), g.state()
    g.close()

    def continue_with(zeta):
        o = Oracle(s, _cfg(s, zeta, 800.0))
        o.set_walkers(*walkers)
        o.set_state(state)
        nw = []
        for _ in range(400):
            r = o.run_report()
            assert r.error_flags == 0
            nw.append(r.nparticles[0])
        o.close()
        return np.array(nw[200:])

    # critical damping draws the population to the new target...
    forced = continue_with(0.04 ** 2 / 4)
    assert abs(forced.mean() - 800.0) < 0.2 * 800.0, forced.mean()
    # ...while the damping term alone only holds the growth rate at zero
    free = continue_with(0.0)
    assert free.mean() > 2.0 * 800.0, free.mean()


def test_forcing_options():
    q = dict(tau=0.01, init_pop=10, mc_cycles=10, nreports=1, shift_damping=0.04)
    assert calc.harmonic_forcing(dict(q, shift_harmonic_crit_damp=True)) == 0.04 ** 2 / 4
    # init_qmc copies a bare shift_harmonic_forcing only when its state already holds a
    # non-zero value, which it never does there: no forcing, as in the reference
    assert calc.harmonic_forcing(dict(q, shift_harmonic_forcing=0.3)) == 0.0
    s = systems.hubbard_k([[4, 0], [0, 4]], 10, U=4.0)
    cfg = calc.config_from_options(s, dict(q, shift_harmonic_crit_damp=True, shift_harmonic_forcing_two_stage=True))
    assert cfg.shift_harmonic_forcing == 0.04 ** 2 / 4


def test_reference_target_switches_on_the_reference_population():
    """reference_target (src/energy_evaluation.F90:638-650): the shift starts to
    vary at the first report whose averaged reference population exceeds the
    target, whatever the total population."""
    s = _hubbard()
    q = dict(tau=0.01, init_pop=1000, mc_cycles=10, nreports=1, reference_target=900.0)
    cfg = calc.config_from_options(s, q)
    assert cfg.target_reference == 1 and cfg.target_particles == 900.0
    o = Oracle(s, cfg)
    o.initial_distribution()
    switched = None
    for k in range(200):
        r = o.run_report()
        if r.vary_shift[0]:
            switched = (k, r)
            break
        assert r.D0_population[0] <= 900.0
    assert switched is not None
    k, r = switched
    assert r.D0_population[0] > 900.0
    assert r.nparticles[0] > 900.0  # the total population passed the target well before
    o.close()
    import pytest
    with pytest.raises(ValueError):
        calc.config_from_options(s, dict(q, target_population=5.0))
