"""Reference-format output files (Write_files) from the host-side results writer: layout of every
record as the reference's edit descriptors give it, and every column against the oracle's
restatement of the per-configuration finalisation, Collect_data and Write_files."""
import os
import re

import numpy as np
import pytest

_F24 = r"(?:  \d| -\d)\.\d{16}E[+-]\d{2}"  # ES24.16: 24 columns
ES24 = re.compile(r"^ " + _F24 + r"(?: " + _F24 + r")*$")
E12 = r"(0|-)\.\d{6}E[+-]\d{2}"


def _sums(rng, nrep):
    s = np.abs(rng.normal(0.5, 0.2, (nrep, 22)))
    s[:, 0] = rng.normal(0, 0.3, nrep)           # mag may be negative
    s[:, 4] = -np.abs(rng.normal(380, 5, nrep))  # en
    s[:, 5] = s[:, 4] ** 2 / 100 + np.abs(rng.normal(5, 1, nrep))
    s[:, 16] = rng.normal(0, 0.1, nrep)          # nbar
    s[:, 20] = -4.0 + rng.normal(0, 0.01, nrep)
    s[:, 21] = -3.9 + rng.normal(0, 0.01, nrep)
    return s


def _floats(line):
    return [float(x.replace("-.", "-0.")) for x in line.split()]


def _load(path, skip_header=True):
    rows = []
    with open(path) as f:
        lines = f.read().splitlines()
    started = not skip_header
    for ln in lines:
        if not started:
            if ln.startswith("    T ") or ln.startswith(" iconf") or ln.startswith(" pair") \
                    or ln.startswith(" T  BIN"):
                started = True
            continue
        if ln.startswith(" replicas_visiting"):
            continue
        rows.append(ln)
    return rows


@pytest.fixture(scope="module")
def written(tmp_path_factory, oracle):
    import j1j2cuda as jc
    rng = np.random.default_rng(3)
    L, H, nrep, nconf, nmess, bins = 8, 4, 5, 3, 200, 6
    temps = np.linspace(8.0, 11.5, nrep)
    res = jc.Results(L, H, temps, nconf=nconf, neq=100, nmess=nmess, bins=bins, pp=0.05,
                     write_numflips=True, write_phitable=True)
    sums, nms, noccs = [], [], []
    for k in range(nconf):
        s = _sums(rng, nrep)
        nm = np.full(nrep, nmess, np.int64)
        nocc = L * L * H - 3 * k
        hist = rng.integers(0, 40, (nrep, bins)).astype(np.float64)
        flips = rng.integers(0, 9, (nrep, L * L * H)).astype(np.int32)
        res.add_conf((s, nm), nocc, np.full(nrep - 1, 1000), np.arange(nrep - 1) * 100 + 50, k,
                     hist, np.full(nrep, -4.5), np.full(nrep, 0.05), flips,
                     np.linspace(-2, 2, L * L * H))
        sums.append(s)
        nms.append(nm)
        noccs.append(nocc)
    d = tmp_path_factory.mktemp("cf")
    res.write(str(d))
    res.close()
    return d, oracle.results_ref(sums, nms, noccs, temps), temps


def test_every_file_is_written(written):
    d, _, _ = written
    names = sorted(os.listdir(d))
    assert names == sorted(f"{s}00080004.dat" for s in ("cfen", "cfma", "cfnm", "cfst", "cfhs",
                                                        "cfxy", "cfnd", "cfnu", "cfpt", "cfph"))


def test_header_records_in_list_directed_layout(written):
    d, _, _ = written
    lines = open(os.path.join(d, "cfen00080004.dat")).read().splitlines()
    assert lines[0] == " program J1J2_6          "
    assert lines[1] == " linear system size                 8"
    assert lines[2] == " J1                         1.0000000000000000     "
    assert lines[4] == " J2                        -1.0000000000000000     "
    assert lines[6] == " phi, xi                        2.0000000000000000        3.0000000000000000     "
    assert lines[7] == " impurity conc.             5.0000000000000003E-002"
    assert lines[11] == " sampler mode            PT   "
    assert " disorder configurations processed            3" in lines


@pytest.mark.parametrize("stem,fmt", [("cfen", "es24"), ("cfma", "e12"), ("cfnm", "e12"),
                                      ("cfst", "e12")])
def test_averages_match_the_restatement(written, stem, fmt):
    d, ref, _ = written
    rows = _load(os.path.join(d, f"{stem}00080004.dat"))
    exp = ref[stem]
    assert len(rows) == exp.shape[0]
    for ln, e in zip(rows, exp):
        if fmt == "es24":
            assert ES24.match(ln), ln
            # 16 digits; the error columns difference nearly equal numbers (1e-13 relative)
            np.testing.assert_allclose(_floats(ln), e, rtol=1e-12, atol=1e-300)
        else:
            assert re.fullmatch(r" " + r" ".join([E12] * len(e)), ln), ln
            np.testing.assert_allclose(_floats(ln), e, rtol=6e-6, atol=1e-99)


@pytest.mark.parametrize("stem,ncol", [("cfxy", 10), ("cfnd", 7)])
def test_per_configuration_files(written, stem, ncol):
    d, ref, _ = written
    rows = _load(os.path.join(d, f"{stem}00080004.dat"))
    assert len(rows) == len(ref[stem])
    for ln, e in zip(rows, ref[stem]):
        assert re.fullmatch(r"[ \d]{4}" + (" " + E12) * (ncol - 1), ln), ln
        v = _floats(ln)
        assert v[0] == e[0]
        np.testing.assert_allclose(v[1:], e[1:], rtol=6e-6, atol=1e-99)


def test_pt_histogram_flips_and_phi_files(written):
    d, _, temps = written
    pt = open(os.path.join(d, "cfpt00080004.dat")).read().splitlines()
    assert pt[1] == "   1 0.800000E+01 0.887500E+01         3000          150 0.500000E-01"
    assert pt[-1] == " replicas_visiting_both_extremes            3  0.20000000000000001     "
    hs = _load(os.path.join(d, "cfhs00080004.dat"))
    assert len(hs) == len(temps) * 5  # BINS - 1 records per temperature
    assert re.fullmatch(r" " + E12 + r"    1 " + E12 + " " + E12, hs[0])
    nu = _load(os.path.join(d, "cfnu00080004.dat"))
    assert len(nu) == 3 * len(temps) * 256 and re.fullmatch(r"   1 " + E12 + r" +0 +\d+", nu[0])
    ph = _load(os.path.join(d, "cfph00080004.dat"))
    assert len(ph) == 3 * 256 and ph[0] == "   1        0 -.200000E+01"
