"""C++ host layer without a GPU: the native input reader (tdbem_run
--parse-only) against the Python parser on every golden input, the
WriteGH text format, and the reader's error path."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden, load_mrt_golden, mrt_golden_cases

RUN = os.path.join(ROOT, "td-bem_gb300", "_build", "tdbem_run")


@pytest.fixture(scope="module")
def built():
    import build as b
    b.build()
    from tdbem import lib
    return lib


def summary(m):
    x = m.coords.reshape(-1)
    csum = float(sum(x[i] * (1 + i % 7) for i in range(len(x))))
    e = m.ien.reshape(-1)
    isum = int(sum(int(e[i]) * (1 + i % 5) for i in range(len(e))))
    bsum = float(sum((d + 1) * v for d, v in zip(m.ubc_dofs, m.ubc_vals)) +
                 sum((d + 1) * v for d, v in zip(m.fbc_dofs, m.fbc_vals)))
    return m.nnd, m.nel, m.etype, m.numstep, m.dt, m.nq, m.if_ext, m.E, m.nu, m.rho, \
        len(m.ubc_dofs), len(m.fbc_dofs), csum, isum, bsum


@pytest.mark.parametrize("name", golden_cases())
def test_native_reader_matches_python_parser(built, name, tmp_path):
    z, m = load_golden(name)
    p = tmp_path / "input.txt"
    p.write_text(str(z["input_text"]))
    r = subprocess.run([RUN, str(p), "--parse-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    tok = r.stdout.split()
    vals = dict(zip(tok[0::2], tok[1::2]))
    ref = summary(m)
    keys = ["nnd", "nel", "etype", "numstep", "dt", "nq", "if_ext", "E", "nu", "rho", "ubc",
            "fbc", "coordsum", "iensum", "bcsum"]
    for k, v in zip(keys, ref):
        got = float(vals[k])
        assert got == pytest.approx(v, rel=1e-13, abs=1e-12), k


@pytest.mark.parametrize("name", mrt_golden_cases())
@pytest.mark.parametrize("region", [1, 2])
def test_native_reader_two_region_inputs(built, name, region, tmp_path):
    """formulation = 3 inputs: interface lists and the auxiliary mesh keywords."""
    z, m1, m2 = load_mrt_golden(name)
    m = (m1, m2)[region - 1]
    p = tmp_path / "input.txt"
    p.write_text(str(z[f"input_text_{region}"]))
    r = subprocess.run([RUN, str(p), "--parse-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    tok = r.stdout.split()
    vals = dict(zip(tok[0::2], tok[1::2]))
    for k, v in zip(["nnd", "nel", "numstep", "dt", "E", "coordsum", "iensum", "bcsum"],
                    [summary(m)[i] for i in (0, 1, 3, 4, 7, 12, 13, 14)]):
        assert float(vals[k]) == pytest.approx(v, rel=1e-13, abs=1e-12), k
    assert int(vals["formulation"]) == 3
    assert int(vals["ninterface"]) == len(m.interface)
    assert int(vals["ifsum"]) == sum((int(n) + 1) * (1 + i % 3) for i, n in enumerate(m.interface))
    assert int(vals["nnd_aux"]) == len(m.coords_aux)
    assert int(vals["nel_aux"]) == len(m.ien_aux)
    e = m.ien_aux.reshape(-1)
    assert int(vals["auxsum"]) == sum(int(e[i]) * (1 + i % 5) for i in range(len(e)))


def test_reader_rejects_aux_keywords_outside_multiregion(built, tmp_path):
    """InputT reads the auxiliary mesh only when formulation = 3 (InputT.cpp:117-122)."""
    p = tmp_path / "bad.txt"
    p.write_text("numstep=3;\nnnd_aux=4;\n")
    r = subprocess.run([RUN, str(p), "--parse-only"], capture_output=True, text=True)
    assert r.returncode == 1 and "unaccepted key word nnd_aux" in r.stderr
    from tdbem import inputfile
    with pytest.raises(inputfile.InputError):
        inputfile.parse("numstep=3;\nnnd_aux=4;\n")


def test_reader_rejects_unknown_keyword(built, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("numstep=3;\nbogus=1;\n")
    r = subprocess.run([RUN, str(p), "--parse-only"], capture_output=True, text=True)
    assert r.returncode == 1 and "unaccepted key word bogus" in r.stderr


def test_write_gh_format(built, tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((3, 5)) * 10.0 ** rng.integers(-8, 8, (3, 5))
    a[0, 0] = 0.0
    a[1, 2] = -0.0
    prefix = str(tmp_path / "G1_step")
    built.write_gh(prefix, 7, a)
    text = open(prefix + "7.txt").read().splitlines()
    assert len(text) == 3
    for i, line in enumerate(text):
        assert line == "".join("%15.5e" % v for v in a[i])  # setw(15) setprecision(5) scientific
    back = np.loadtxt(prefix + "7.txt")
    assert np.allclose(back, a, rtol=1e-5, atol=0)
