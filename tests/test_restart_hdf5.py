"""HANDE restart files (src/restart_hdf5.F90) without an HDF5 library:
hande_gb300.hdf5lite reads and writes the file format subset HANDE uses, and
hande_gb300.restart maps a restart onto a calculation.  Pinned against HANDE's
own restart files (reduced to tests/golden/restart_*.npz by
tests/golden/make_restart_golden.py):
- K_ii = H_ii - H_00 that HANDE stored for each of its determinants equals the
  oracle's diagonal element of the same determinant after the 32- to 64-bit
  word conversion: 4580 determinants of an 18-site Hubbard model and 141 of
  He2 aug-cc-pVDZ (which also rescales integer populations to real-amplitude
  fixed point);
- files written here have the header messages of HANDE's (golden structure)
  and read back unchanged;
- a calculation restarted from them continues on the oracle."""

import json
import os

import numpy as np
import pytest

from hande_gb300 import hdf5lite, restart, systems
from hande_gb300._abi import make_config
from oracle.pyoracle import Oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _hubbard():
    return systems.hubbard_k([[3, 3], [3, -3]], 18, U=0.5)


def _he2():
    return systems.read_in(os.path.join(GOLDEN, "He2-aug-cc-pVDZ.fcidump"), nel=4, ms=0)


def test_word_conversion():
    # bit_string_32_to_64: pairs of 32-bit words, low first; an odd count clears the high half
    w32 = np.array([[-1, 5, 7], [1, 0, -2]], dtype=np.int32)
    out = restart._words64(w32, 32, 96, 0)
    assert out.dtype == np.int64 and out.shape == (2, 2)
    assert out[0, 0] == np.int64((5 << 32) | 0xFFFFFFFF)
    assert out[0, 1] == 7
    assert out[1, 0] == 1 and out[1, 1] == 0xFFFFFFFE
    # 64-bit words pass through; information-string words are dropped
    w64 = np.array([[3, 9, 42]], dtype=np.int64)
    assert restart._words64(w64, 64, 128, 1).tolist() == [[3, 9]]


def test_population_rescaling():
    p = np.array([[7], [-7], [0]], dtype=np.int64)
    assert restart._rescale(p, 1, 1 << 31).ravel().tolist() == [7 << 31, -(7 << 31), 0]
    # integer division toward zero, as Fortran's
    assert restart._rescale(p, 4, 1).ravel().tolist() == [1, -1, 0]


@pytest.mark.parametrize("name,make", [("restart_hubbard_k_2d", _hubbard), ("restart_he2", _he2)])
def test_kii_of_hande_restart_matches_oracle(name, make):
    g = _golden(name)
    s = make()
    cfg = make_config(s, tau=0.01, real_amplitudes=bool(g["real_factor"][0] > 1), state_size=20000,
                      spawned_state_size=20000)
    o = Oracle(s, cfg)
    ref = g["reference"]
    assert int(ref[0]) == int(cfg.ref_det[0])
    e0 = o.sc0(ref)
    got = np.array([o.sc0(f) - e0 for f in g["states"]])
    np.testing.assert_allclose(got, g["kii"], rtol=1e-12, atol=1e-12)
    # the list: sorted in HANDE's order, unique, every determinant with nel electrons
    u = g["states"].view(np.uint64)[:, 0]
    assert np.all(u[1:] > u[:-1])
    assert all(bin(int(x)).count("1") == s.nel for x in u)
    # total population = sum |N_i| in walker units
    rf = int(g["real_factor"][0])
    assert abs(np.abs(g["pops"]).sum() / rf - g["nparticles_old"][0]) < 1e-6 * g["nparticles_old"][0] + 1.0
    o.close()


def _write(path, g, **kw):
    restart.write(path, g["states"], g["pops"], g["kii"], nbasis=kw.get("nbasis", 36),
                  real_factor=int(g["real_factor"][0]), iteration=int(g["iteration"][0]), shift=g["shift"],
                  vary_shift=g["vary_shift"], nparticles_old=g["nparticles_old"], reference=g["reference"],
                  mtime=1_700_000_000)


def test_written_restart_reads_back_and_has_hande_structure(tmp_path):
    g = _golden("restart_hubbard_k_2d")
    path = str(tmp_path / "HANDE.RS.4.p0.H5")
    _write(path, g)
    r = restart.read(restart.restart_paths(4, str(tmp_path)), 36, 1, 1)
    np.testing.assert_array_equal(r["states"], g["states"])
    np.testing.assert_array_equal(r["pops"], g["pops"])
    np.testing.assert_array_equal(r["kii"], g["kii"])
    assert r["iteration"] == int(g["iteration"][0]) and r["shift"] == list(g["shift"])
    assert r["vary_shift"] == list(g["vary_shift"]) and r["nparticles_old"] == list(g["nparticles_old"])
    assert r["restart_version"] == restart.RESTART_VERSION
    # every object HANDE's files share with ours carries the same header messages
    golden = json.load(open(os.path.join(GOLDEN, "restart_structure.json")))
    ours = {k: [list(m) for m in v] for k, v in hdf5lite.structure(path).items()}
    for version in ("version2_fciqmc", "version3"):
        common = set(golden[version]) & set(ours)
        assert len(common) >= 25, version
        for k in common:
            assert ours[k] == golden[version][k], (version, k)
    # the datasets read_restart_hdf5 reads without checking that they exist
    d = hdf5lite.read(path)
    for k in ("/metadata/nprocs", "/metadata/restart version", "/metadata/i0_length", "/metadata/calc type",
              "/metadata/uuid", "/qmc/psips/determinants", "/qmc/psips/populations", "/qmc/psips/data",
              "/qmc/psips/total population", "/qmc/state/ncycles", "/qmc/state/shift",
              "/qmc/state/projected energy", "/qmc/state/projected energy real",
              "/qmc/state/projected energy imag", "/qmc/reference/reference determinant",
              "/qmc/reference/Hilbert space reference determinant",
              "/qmc/reference/reference population @ t-1", "/qmc/reference/reference population @ t-1 real",
              "/qmc/reference/reference population @ t-1 imag"):
        assert k in d, k
    assert d["/qmc/psips/determinants"].dtype == np.int64 and int(d["/metadata/i0_length"]) == 64


def test_hdf5_writer_general_shapes(tmp_path):
    # more members than one symbol-table node holds, scalars, strings, an empty dataset
    ds = {"/g/x%02d" % i: np.arange(i, dtype=np.int32) for i in range(20)}
    ds["/s"] = b"text"
    ds["/f"] = np.float64(2.5)
    ds["/h/nested/u"] = np.array([[1, 2], [3, 4]], dtype=np.int64)
    path = str(tmp_path / "t.h5")
    hdf5lite.write(path, ds, groups=["/empty"])
    back = hdf5lite.read(path)
    assert set(back) == set(ds)
    for k, v in ds.items():
        if isinstance(v, bytes):
            assert back[k].item() == v
        else:
            np.testing.assert_array_equal(back[k], np.asarray(v))
            assert back[k].dtype == np.asarray(v).dtype


def test_restart_continues_on_oracle(tmp_path):
    g = _golden("restart_hubbard_k_2d")
    _write(str(tmp_path / "HANDE.RS.0.p0.H5"), g)
    s = _hubbard()
    cfg = make_config(s, tau=0.01, ncycles=25, seed=7, target_population=5500, state_size=40000,
                      spawned_state_size=40000)
    paths = restart.restart_paths(0, str(tmp_path))
    assert restart.reference_of(paths, s) == list(range(18))
    o = Oracle(s, cfg)
    r = restart.load_into(o, paths)
    st = o.state()
    assert st.iteration == r["iteration"] and st.vary_shift[0] == 1
    assert st.shift[0] == r["shift"][0]
    n0 = g["nparticles_old"][0]
    for _ in range(2):
        rep = o.run_report()
        assert rep.error_flags == 0
    assert rep.iteration == r["iteration"] + 50
    assert 0.5 * n0 < rep.nparticles[0] < 2.0 * n0
    assert np.isfinite(rep.shift[0])
    # and is written back as a restart file of its own
    out = str(tmp_path / "HANDE.RS.1.p0.H5")
    restart.save_from(o, out, report=rep.as_dict(1), mtime=1_700_000_000)
    back = restart.read([out], s.nbasis, 1, 1)
    st2, po2, da2 = o.walkers()
    # a calculation around another reference refuses the file
    other = Oracle(s, make_config(s, tau=0.01, state_size=40000, spawned_state_size=40000,
                                  reference=list(range(17)) + [19]))
    with pytest.raises(ValueError):
        restart.load_into(other, paths)
    other.close()
    np.testing.assert_array_equal(back["states"], st2)
    np.testing.assert_array_equal(back["pops"], po2)
    assert back["iteration"] == rep.iteration
    o.close()


REF_SUITE = "/root/reference/test_suite"


@pytest.mark.skipif(not os.path.isdir(REF_SUITE), reason="HANDE's test suite is not present")
def test_reader_opens_every_hande_file():
    import glob
    import re
    files = sorted(glob.glob(os.path.join(REF_SUITE, "**", "*.H5"), recursive=True))
    assert len(files) >= 40
    sets = {}
    for p in files:
        d = hdf5lite.read(p)
        m = re.match(r"(.*)/HANDE\.RS\.(\d+)\.p(\d+)\.H5$", p)
        if m:
            n = d["/qmc/psips/determinants"].shape[0]
            assert d["/qmc/psips/populations"].shape[0] == n and d["/qmc/psips/data"].shape[0] == n, p
            sets.setdefault((m.group(1), m.group(2)), []).append(d)
    assert len(sets) >= 20
    for (directory, rid), ds in sets.items():
        i0 = int(ds[0]["/metadata/i0_length"])
        info = int(ds[0]["/basis/info string len"]) if "/basis/info string len" in ds[0] else 0
        nbasis = int(ds[0]["/basis/nbasis"]) if "/basis/nbasis" in ds[0] else 0
        nw = (nbasis + i0 - 1) // i0 if nbasis else ds[0]["/qmc/psips/determinants"].shape[1] - info
        counts = set()
        tot = 0.0
        for d in ds:
            w = np.ascontiguousarray(d["/qmc/psips/determinants"][:, :nw])
            w = w.view(np.uint64) if i0 == 64 else w.astype(np.int64) & 0xFFFFFFFF
            counts |= {sum(bin(int(x)).count("1") for x in row) for row in w}
            scale = int(d["/qmc/psips/population scale factor"][0]) if "/qmc/psips/population scale factor" in d else 1
            tot += np.abs(d["/qmc/psips/populations"][:, 0].astype(np.float64)).sum() / scale
        # one electron count per calculation (CCMC excitors carry no fixed count)
        if "/metadata/calc type" in ds[0] and int(ds[0]["/metadata/calc type"]) == 4:
            assert len(counts) == 1, (directory, rid, counts)
            want = float(np.ravel(ds[0]["/qmc/psips/total population"])[0])
            # complex populations: the first column is the real part only
            if ds[0]["/qmc/psips/populations"].shape[1] == 1:
                assert abs(tot - want) <= 1e-6 * want + 1.0, (directory, rid, tot, want)


def continue_and_compare(make_calc, tmp_path, nreports):
    """Continue HANDE's Hubbard restart with HANDE's parameters for nreports
    reports, reblock after the same 10-report window, and compare with HANDE's
    own continuation (tests/golden/restart_continuation.json).  The streams
    differ (HANDE's dSFMT, Philox here), so the comparison is statistical: the
    projected energy within 3 combined standard errors.  The shift is held to
    5: its reblocked error understates its spread on this system.  HANDE's own
    run of the same calculation from scratch (the run that wrote the restart)
    gives -0.0480(10) or -0.0491(8) depending on the window, and its
    continuation -0.0482(2); the oracle's runs give -0.0496(4) and -0.0491(4)
    after restarts, -0.0492(8) from scratch, with projected energies that agree
    with HANDE's to 1e-5."""
    from hande_gb300 import analysis
    cont = json.load(open(os.path.join(GOLDEN, "restart_continuation.json")))
    q = cont["qmc"]
    g = _golden("restart_hubbard_k_2d")
    _write(str(tmp_path / "HANDE.RS.0.p0.H5"), g)
    s = _hubbard()
    cfg = make_config(s, tau=q["tau"], ncycles=q["ncycles"], seed=q["rng_seed"],
                      target_population=q["target_particles"], shift_damping=q["shift_damping"],
                      state_size=60000, spawned_state_size=60000)
    c = make_calc(s, cfg)
    r0 = restart.load_into(c, restart.restart_paths(0, str(tmp_path)))
    assert r0["iteration"] == cont["first_iteration"]
    shift, num, d0 = [], [], []
    for _ in range(nreports):
        rep = c.run_report()
        assert rep.error_flags == 0
        shift.append(rep.shift[0])
        num.append(rep.proj_energy[0])
        d0.append(rep.D0_population[0])
    c.close()
    k0 = cont["reference_stats"]["first_report"]
    S, Serr, _ = analysis.mean_error(shift[k0:])
    E, Eerr, _ = analysis.projected_energy(num[k0:], d0[k0:])
    ref = cont["reference_stats"]
    zE = (E - ref["proj_energy"]) / np.hypot(Eerr, ref["proj_energy_error"])
    zS = (S - ref["shift"]) / np.hypot(Serr, ref["shift_error"])
    msg = "E_proj %.6f(%.6f) vs HANDE %.6f(%.6f), z=%.2f; shift %.5f(%.5f) vs %.5f(%.5f), z=%.2f" % (
        E, Eerr, ref["proj_energy"], ref["proj_energy_error"], zE, S, Serr, ref["shift"], ref["shift_error"], zS)
    print(msg)
    assert abs(zE) < 3.0, msg
    assert abs(zS) < 5.0, msg


def test_oracle_continues_hande_restart_like_hande(tmp_path):
    continue_and_compare(lambda s, cfg: Oracle(s, cfg), tmp_path, 400)


def test_driver_vary_shift_option_overrides_restart(tmp_path, monkeypatch):
    """qmc.vary_shift (init_estimators, src/qmc.F90:881-893) overrides the
    restart's vary shift, and a shift that does not vary restarts from
    initial_shift; the fciqmc driver's host logic, run with the oracle in the
    engine's place."""
    from hande_gb300 import calc

    class OracleEngine(Oracle):
        def get_state(self):
            return self.state()

    monkeypatch.setattr(calc, "Engine", OracleEngine)
    g = _golden("restart_hubbard_k_2d")
    _write(str(tmp_path / "HANDE.RS.0.p0.H5"), g)
    # a target the population never reaches: the switch at a report's end stays out of play
    qmc = dict(tau=0.01, rng_seed=7, init_pop=10, mc_cycles=25, nreports=2, target_population=1e9,
               state_size=40000, spawned_state_size=40000, initial_shift=-0.25)
    res = calc.fciqmc(_hubbard(), dict(qmc, vary_shift=False), restart={"read": 0}, directory=str(tmp_path),
                      verbose=False)
    for rep in res["reports"]:
        assert rep["vary_shift"] == [0] and rep["Shift"] == [-0.25]
    res["engine"].close()
    res = calc.fciqmc(_hubbard(), qmc, restart={"read": 0}, directory=str(tmp_path), verbose=False)
    assert res["reports"][0]["vary_shift"] == [1]
    assert res["reports"][0]["Shift"][0] != -0.25
    res["engine"].close()
