"""Drop-in driver: input parsing, Fortran output formats (CPU) and an end-to-end run (GPU)."""
from __future__ import annotations

import os

import numpy as np
import pytest

INPUT = """sys_name
  'tiny'

acell
  6.0d0

NB
  2
NBocc
  2
NG
  16
  128
NK
  2

Nscf
  2
NCG
  2
dt
  0.005
NT
  8
Nomega
  50
omegaM
  2.0
field_option
  'LP'
omegac
  1.55
Tpulse
  0.05
E0
  20.0
nenvelope
  2
atoms
  1             : Nspecies
  2             : Zeff
  1.0d0         : alpha
  1             : Nion
  0.5d0  1      : Rion, Kion
"""


def test_read_input_first_value_and_atoms(tmp_path):
    from mattohf_gb300 import read_input
    from oracle import mattohf_oracle as O
    p = tmp_path / "input.dat"
    p.write_text(INPUT)
    cfg = read_input(str(p))
    assert (cfg.NG, cfg.NK, cfg.NB, cfg.NBocc, cfg.NT) == (16, 2, 2, 2, 8)   # first value only
    assert cfg.sys_name == "tiny" and cfg.field_option == "LP"
    assert cfg.Zeff == [2.0] and cfg.Rion == [0.5] and cfg.Kion == [1]
    o = O.read_input(str(p))
    for k in ("acell", "NG", "NK", "NB", "NBocc", "Nscf", "NCG", "dt", "NT", "Nomega", "omegaM",
              "omegac", "Tpulse", "E0", "nenvelope", "Zeff", "alpha", "Rion", "Kion", "sys_name"):
        assert getattr(cfg, k) == getattr(o, k), k


def test_fortran_e_format():
    from mattohf_gb300.driver import fortran_e
    assert fortran_e(1.0) == "  0.100000000000E+01"
    assert fortran_e(-0.00123456789012345) == " -0.123456789012E-02"
    assert fortran_e(0.0) == "  0.000000000000E+00"
    assert fortran_e(9.9999999999999e5) == "  0.100000000000E+07"
    assert fortran_e(1.5e123) == "  0.150000000000+124"
    assert fortran_e(2.5, e=3) == " 0.250000000000E+001"


def test_define_afield_matches_oracle():
    from mattohf_gb300 import RunConfig, define_afield
    from oracle import mattohf_oracle as O
    import dataclasses
    cfg = RunConfig(NT=300, dt=0.05, field_option="LP", omegac=1.55, Tpulse=5.0, E0=2.0, nenvelope=4,
                    phiCEP=0.3)
    t, A, Aave, E = define_afield(cfg)
    ot, oA, oAave, oE, _ = O.define_afield(O.Config(**{f.name: getattr(cfg, f.name) for f in dataclasses.fields(O.Config)}))
    assert np.array_equal(A, oA) and np.array_equal(Aave, oAave) and np.array_equal(E, oE)


@pytest.mark.gpu
def test_driver_end_to_end(tmp_path, built_lib):
    from mattohf_gb300 import read_input
    from mattohf_gb300.driver import run
    p = tmp_path / "input.dat"
    p.write_text(INPUT)
    cfg = read_input(str(p))
    res = run(cfg, out_dir=str(tmp_path), log=lambda *a: None)
    for f in ("potential.out", "vk.out", "tiny_GSinfo.out", "tiny_DoS.out", "tiny_band.out",
              "tiny_EtotNJEAt.out", "tiny_JEAF.out", "tiny_JEAF_window.out", "tiny_dipole.out"):
        assert os.path.exists(tmp_path / f), f
    rows = [l for l in open(tmp_path / "tiny_EtotNJEAt.out") if not l.startswith("#")]
    assert len(rows) == cfg.NT and len(rows[0]) == 8 * 20 + 1
    vals = np.array([[float(l[i * 20:(i + 1) * 20].replace("E", "e")) for i in range(8)] for l in rows])
    assert np.allclose(vals[:, 1], res["Etot"], rtol=1e-11, atol=0)
    # the dipole extension: -int J dt by the trapezoid rule from the initial current
    from oracle import mattohf_oracle as O
    prow = [l for l in open(tmp_path / "tiny_dipole.out") if not l.startswith("#")]
    P = np.array([float(l[20:40].replace("E", "e")) for l in prow])
    assert len(prow) == cfg.NT
    Pref = O.dipole_from_current(res["time"], res["Je"], res["J0"], cfg.dt)
    assert np.allclose(P, Pref, rtol=1e-11, atol=1e-13 * np.max(np.abs(Pref)))
    assert np.allclose(res["P"], Pref, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_fourier_matches_oracle(built_lib):
    from mattohf_gb300 import RunConfig
    from mattohf_gb300.driver import fourier
    from oracle import mattohf_oracle as O
    import dataclasses
    cfg = RunConfig(dt=0.1, NT=400, Nomega=64, omegaM=3.0, field_option="LP", Tpulse=5.0)
    rng = np.random.default_rng(0)
    t = cfg.dt * np.arange(cfg.NT)
    J, E, A = rng.standard_normal((3, cfg.NT))
    oc = O.Config(**{f.name: getattr(cfg, f.name) for f in dataclasses.fields(O.Config)})
    w, JF, EF, AF, _, _ = O.fourier_tr(oc, t, J, 0.3, E, A)
    ft = fourier(cfg, t, J, 0.3, E, A, window=False)
    assert np.allclose(ft[:, 0], w, rtol=1e-15)
    for col, ref in ((1, JF), (3, EF), (5, AF)):
        assert np.max(np.abs(ft[:, col] + 1j * ft[:, col + 1] - ref)) <= 1e-12 * np.max(np.abs(ref))
    w2, JF2, _, _ = O.window_fourier_tr(oc, t, J, 0.3, E, A)
    fw = fourier(cfg, t, J, 0.3, E, A, window=True)
    assert np.max(np.abs(fw[:, 1] + 1j * fw[:, 2] - JF2)) <= 1e-12 * np.max(np.abs(JF2))
    # a time grid that is not uniform takes a sincos per term instead of the
    # rotation recurrence; longer series span several time chunks
    for tt in (t + 1e-3 * rng.standard_normal(cfg.NT), None):
        if tt is None:
            cfg2 = dataclasses.replace(cfg, NT=3000)
            tt = cfg2.dt * np.arange(cfg2.NT)
            J3, E3, A3 = rng.standard_normal((3, cfg2.NT))
        else:
            cfg2, J3, E3, A3 = cfg, J, E, A
        oc2 = O.Config(**{f.name: getattr(cfg2, f.name) for f in dataclasses.fields(O.Config)})
        _, JF3, EF3, AF3, _, _ = O.fourier_tr(oc2, tt, J3, 0.3, E3, A3)
        f3 = fourier(cfg2, tt, J3, 0.3, E3, A3, window=False)
        for col, ref in ((1, JF3), (3, EF3), (5, AF3)):
            assert np.max(np.abs(f3[:, col] + 1j * f3[:, col + 1] - ref)) <= 1e-12 * np.max(np.abs(ref))


# ---------------------------------------------------------------------------
# C++ drop-in driver (mattohf_gb300/_lib/mattohf, built by build())
# ---------------------------------------------------------------------------
def _cpp_driver():
    from mattohf_gb300 import build
    build.build()
    return build.DRIVER


def _run_cpp(name_line: str, out_dir, cwd):
    import subprocess
    return subprocess.run([_cpp_driver(), str(out_dir)], input=name_line + "\n", capture_output=True, text=True,
                          cwd=str(cwd), timeout=600)


def test_cpp_driver_rejects_missing_input(tmp_path):
    r = _run_cpp("'no_such_input.dat'", tmp_path, tmp_path)
    assert r.returncode == 1
    assert "cannot open input file 'no_such_input.dat'" in r.stderr


def test_cpp_driver_rejects_bad_integer(tmp_path):
    (tmp_path / "bad.dat").write_text("NG\n  1.5x\n")
    r = _run_cpp('"bad.dat"', tmp_path, tmp_path)
    assert r.returncode == 1
    assert "bad integer value '1.5x'" in r.stderr


def _numbers(path):
    """Every number in a file, in order (headers are identical in both drivers' files)."""
    import re
    num = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")
    return np.array([float(t) for line in open(path) for t in num.findall(line)])


@pytest.mark.gpu
@pytest.mark.parametrize("field", ["LP", "LR"])
def test_cpp_driver_matches_python_driver(tmp_path, built_lib, field):
    """Every output file of the C++ driver against the Python driver on the same input."""
    from mattohf_gb300 import read_input
    from mattohf_gb300.driver import run
    text = INPUT.replace("'LP'", f"'{field}'")
    (tmp_path / "input.dat").write_text(text)
    py_dir, cpp_dir = tmp_path / "py", tmp_path / "cpp"
    py_dir.mkdir()
    cpp_dir.mkdir()
    run(read_input(str(tmp_path / "input.dat")), out_dir=str(py_dir), log=lambda *a: None)
    r = _run_cpp("'input.dat'", cpp_dir, tmp_path)
    assert r.returncode == 0, r.stderr
    files = sorted(os.listdir(py_dir))
    assert files == sorted(os.listdir(cpp_dir))
    assert ("tiny_sigmaeps.out" in files) == (field == "LR")
    for f in files:
        a, b = _numbers(py_dir / f), _numbers(cpp_dir / f)
        assert a.shape == b.shape, f
        # same kernels in the same order; host-side sums (SCF density change,
        # DoS broadening) may round differently from numpy's pairwise sums
        assert np.allclose(a, b, rtol=1e-11, atol=1e-300), f


# ---------------------------------------------------------------------------
# Drivers against the oracle's restatement of the program (oracle/mattohf_program.py)
# ---------------------------------------------------------------------------
_NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+|[-+]\d{3})?"


def _parse(tok: str) -> float:
    import re
    m = re.fullmatch(r"([-+]?(?:\d+\.\d*|\.\d+|\d+))([-+]\d{3})", tok)   # Ew.d with a 3-digit exponent
    return float(m.group(1) + "e" + m.group(2)) if m else float(tok)


def _compare_with_oracle(got_path, ref_path, fixed_width: bool, rtol=1e-8):
    """Same records: for fixed-width (E/F/I edit descriptor) files the text with
    every number masked must be identical (headers, asterisks, Infinity, field
    layout); every number must agree to rtol, with an absolute floor of 1e-11
    of the file's largest finite magnitude."""
    import re
    got = open(got_path).read().splitlines()
    ref = open(ref_path).read().splitlines()
    assert len(got) == len(ref), (got_path, len(got), len(ref))
    gnums, rnums = [], []
    for a, b in zip(got, ref):
        if fixed_width:
            assert re.sub(_NUM, "#", a) == re.sub(_NUM, "#", b), (got_path, a, b)
        else:
            assert len(re.findall(_NUM, a)) == len(re.findall(_NUM, b)), (got_path, a, b)
        gnums += [_parse(t) for t in re.findall(_NUM, a)]
        rnums += [_parse(t) for t in re.findall(_NUM, b)]
    g, r = np.array(gnums), np.array(rnums)
    finite = np.abs(r[np.abs(r) < 1e300])
    floor = 1e-11 * (finite.max() if finite.size else 1.0)
    bad = np.abs(g - r) > rtol * np.abs(r) + floor
    assert not bad.any(), (got_path, g[bad][:5], r[bad][:5])


@pytest.mark.gpu
@pytest.mark.parametrize("field,nb", [("LP", 2), ("LR", 2), ("LP", 3)])
def test_drivers_match_oracle_program(tmp_path, built_lib, field, nb):
    """Every reference output file of the C++ drop-in driver and of the Python
    driver against the file the oracle's restatement of the program writes
    from its own results and the reference's edit descriptors
    (src/GS_calculation.f90:21-118, 239-265; src/RT_calculation.f90:21-65,
    246-351; src/Prep_periodic_ion_potential.f90:23-27;
    src/Initialization.f90:148-155).  With nb = 2 every band is occupied (the
    gap columns of GSinfo take their empty-section values), with nb = 3 one
    band is empty."""
    from mattohf_gb300 import read_input
    from mattohf_gb300.driver import run
    from oracle import mattohf_oracle as O
    from oracle.mattohf_program import run_program
    text = INPUT.replace("'LP'", f"'{field}'").replace("NB\n  2\n", f"NB\n  {nb}\n")
    (tmp_path / "input.dat").write_text(text)
    dirs = {k: tmp_path / k for k in ("oracle", "cpp", "py")}
    for d in dirs.values():
        d.mkdir()
    ocfg = O.read_input(str(tmp_path / "input.dat"))
    assert ocfg.NB == nb
    run_program(ocfg, str(dirs["oracle"]))
    r = _run_cpp("'input.dat'", dirs["cpp"], tmp_path)
    assert r.returncode == 0, r.stderr
    run(read_input(str(tmp_path / "input.dat")), out_dir=str(dirs["py"]), log=lambda *a: None)
    ref_files = sorted(os.listdir(dirs["oracle"]))
    assert ("tiny_sigmaeps.out" in ref_files) == (field == "LR")
    for drv in ("cpp", "py"):
        files = set(os.listdir(dirs[drv]))
        assert files == set(ref_files) | {"tiny_dipole.out"}, (drv, files)   # the dipole is an extension
        for f in ref_files:
            _compare_with_oracle(dirs[drv] / f, dirs["oracle"] / f, fixed_width=f not in ("potential.out", "vk.out"))
