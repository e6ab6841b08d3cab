"""The host side of the calc interface (hande_gb300.calc): HANDE's Lua option
names (src/lua_hande_calc.f90) mapped onto hgpu_config, without a GPU."""

import os

import pytest

from hande_gb300 import calc, systems
from hande_gb300._abi import EXCIT_GEN
from tests.conftest import GOLDEN

QMC = dict(tau=0.01, mc_cycles=10, nreports=5, init_pop=10, rng_seed=3)


def _sys():
    return systems.read_in(os.path.join(GOLDEN, "H2O-RHF-sto-2g.fcidump"))


def test_semi_stoch_table():
    s = _sys()
    cfg = calc.config_from_options(s, QMC, semi_stoch=dict(space="high", size=50, start_iteration=20))
    assert (cfg.semi_stoch_space, cfg.semi_stoch_size, cfg.semi_stoch_start_iter, cfg.semi_stoch_shift_iter) == \
        (1, 50, 20, -1)
    # shift_start_iteration: start_iteration = huge(0), fixed up when the shift varies
    cfg = calc.config_from_options(s, QMC, semi_stoch=dict(space="high", size=50, shift_start_iteration=7))
    assert cfg.semi_stoch_shift_iter == 7 and cfg.semi_stoch_start_iter > 2 ** 40
    cfg = calc.config_from_options(s, QMC, semi_stoch=dict(space="ci", ci_space=dict(ex_level=2)))
    assert (cfg.semi_stoch_space, cfg.semi_stoch_ci_level) == (4, 2)
    cfg = calc.config_from_options(s, QMC)
    assert cfg.semi_stoch_space == 0
    # separate_annihilation = false: combined annihilation
    cfg = calc.config_from_options(s, QMC, semi_stoch=dict(space="high", size=5, separate_annihilation=False))
    assert (cfg.semi_stoch_space, cfg.semi_stoch_combined) == (1, 1)
    cfg = calc.config_from_options(s, QMC, semi_stoch=dict(space="high", size=5))
    assert cfg.semi_stoch_combined == 0
    for bad in (dict(size=5), dict(space="high"), dict(space="read"), dict(space="high", size=5, bogus=1)):
        with pytest.raises(ValueError):
            calc.config_from_options(s, QMC, semi_stoch=bad)


def test_generator_names_and_weights():
    s = _sys()
    for name in ("uniform_power_pitzer", "heat_bath_power_pitzer", "heat_bath_power_pitzer_ref",
                 "uniform_cauchy_schwarz", "heat_bath_cauchy_schwarz", "power_pitzer_orderN",
                 "renorm_spin", "heat_bath"):
        cfg = calc.config_from_options(s, dict(QMC, excit_gen=name, power_pitzer_min_weight=0.05))
        assert cfg.excit_gen == EXCIT_GEN[name]
        assert cfg.power_pitzer_min_weight == 0.05
    assert "power_pitzer" not in EXCIT_GEN  # refused by HANDE for read_in systems
    with pytest.raises(ValueError):
        calc.config_from_options(s, dict(QMC, not_an_option=1))


def test_restart_table(tmp_path):
    s = _sys()
    # keys outside HANDE's restart table, and a read without files, stop before any device work
    with pytest.raises(ValueError):
        calc.fciqmc(s, QMC, restart=dict(read=0, bogus=1), directory=str(tmp_path), verbose=False)
    with pytest.raises(FileNotFoundError):
        calc.fciqmc(s, QMC, restart=dict(read=3), directory=str(tmp_path), verbose=False)
    assert calc._restart_id(True) == 0 and calc._restart_id(5) == 5
    assert calc._restart_id(False) is None and calc._restart_id(None) is None
