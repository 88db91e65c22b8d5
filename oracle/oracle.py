"""ORACLE — test infrastructure only.

ctypes front end of ``liboracle.so`` (the C restatement of the reference hot path and the replay
of the device engine) and of ``_ref/libref_corr3d.so`` (make_corr_rand_3d around the reference's
vendored Ooura FFT).  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
may import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_corr3d.so")
NSUM = 22
SUM_FIELDS = ("mag", "absmag", "mag2", "mag4", "en", "en2", "strx_abs", "stry_abs", "strx2",
              "strx4", "stry2", "stry4", "str2", "str4", "absstr", "nem", "nbar", "nbarabs",
              "nbar2", "nbar4", "best_en", "final_en")

_lib = None
_ref = None


def build(ref: bool = False, reference: str | None = None) -> None:
    """Compile the oracle (and, with ref=True, the Ooura-linked reference from the reference tree
    `reference`, default: beside the repository) with make."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        extra = [f"REFERENCE={reference}"] if reference else []
        subprocess.run(["make", "-s", "-C", HERE, "ref"] + extra, check=True)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Lat(C.Structure):
    _fields_ = [("L", C.c_int32), ("H", C.c_int32), ("N", C.c_int32), ("nimp", C.c_int32),
                ("J1h", C.c_double), ("J1v", C.c_double), ("J2", C.c_double), ("J3", C.c_double),
                ("m", C.POINTER(C.c_int32)), ("occu", C.POINTER(C.c_int8)),
                ("jh", C.POINTER(C.c_int8)), ("jv", C.POINTER(C.c_int8)),
                ("p", C.POINTER(C.c_double))]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
                os.path.getmtime(os.path.join(HERE, f)) for f in ("oracle.c", "oracle.h")):
            build()
        _lib = C.CDLL(LIB_PATH)
        L = _lib
        L.or_kiss_u.restype = C.c_double
        L.or_erfcc.restype = C.c_double
        L.or_erfcc.argtypes = [C.c_double]
        L.or_field_ref.restype = C.c_double
        L.or_nbar_ref.restype = C.c_double
        L.or_dexp.restype = C.c_double
        L.or_dexp.argtypes = [C.c_double]
        L.or_replay_sweeps.restype = C.c_int64
        L.or_setup_vacancies.restype = C.c_int32
        L.or_bench_pt_ref.restype = C.c_double
        L.or_bench_pt_multi.restype = C.c_double
        L.or_wolff_step.restype = C.c_int64
    return _lib


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            build(ref=True)
        _ref = C.CDLL(REF_PATH)
    return _ref


# ----------------------------------------------------------------------------------------------
# KISS05 / gkiss05 / erfcc
# ----------------------------------------------------------------------------------------------
def kiss_draw(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().or_kiss_draw(C.c_int32(seed), C.c_int32(n), _p(out, C.c_double))
    return out


def gkiss_fill(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().or_gkiss_fill(C.c_int32(seed), C.c_int32(n), _p(out, C.c_double))
    return out


def erfcc(x: float) -> float:
    return lib().or_erfcc(float(x))


def dexp(x: float) -> float:
    return lib().or_dexp(float(x))


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.empty(4, np.uint32)
    lib().or_philox(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(out, C.c_uint32))
    return out


# ----------------------------------------------------------------------------------------------
# Lattice model
# ----------------------------------------------------------------------------------------------
class Model:
    """One disorder configuration on an L x L x H lattice, reference conventions."""

    def __init__(self, L, H, p, occu=None, jh=None, jv=None, J1h=1.0, J1v=1.0, J2=-1.0, J3=1.0):
        self.L, self.H = int(L), int(H)
        self.N = self.L * self.L * self.H
        N = self.N
        self.m = neighbors(self.L, self.H)
        self.p = np.ascontiguousarray(p, np.float64).reshape(N)
        self.occu = np.ones(N, np.int8) if occu is None else np.ascontiguousarray(occu, np.int8)
        self.jh = np.ones(N, np.int8) if jh is None else np.ascontiguousarray(jh, np.int8)
        self.jv = np.ones(N, np.int8) if jv is None else np.ascontiguousarray(jv, np.int8)
        self.nimp = int(N - int(self.occu.sum()))
        self.J = (float(J1h), float(J1v), float(J2), float(J3))
        self.lat = Lat(self.L, self.H, N, self.nimp, self.J[0], self.J[1], self.J[2], self.J[3],
                       _p(self.m, C.c_int32), _p(self.occu, C.c_int8), _p(self.jh, C.c_int8),
                       _p(self.jv, C.c_int8), _p(self.p, C.c_double))

    def ref(self):
        return C.byref(self.lat)

    # reference arithmetic --------------------------------------------------------------------
    def field(self, s, i):
        n = C.c_double()
        f = lib().or_field_ref(self.ref(), _p(s, C.c_int8), C.c_int32(i), C.byref(n))
        return f, n.value

    def measurement(self, s):
        out = np.empty(4)
        lib().or_measurement_ref(self.ref(), _p(s, C.c_int8), _p(out, C.c_double))
        return out

    def nbar(self, s):
        return lib().or_nbar_ref(self.ref(), _p(s, C.c_int8))

    def metro_sweep(self, s, beta, obs, kiss_state, rnd=False):
        order = np.empty(self.N, np.int32)
        lib().or_metro_sweep_ref(self.ref(), _p(s, C.c_int8), C.c_double(beta), None,
                                 _p(obs, C.c_double), _p(kiss_state, C.c_uint32),
                                 C.c_int32(int(rnd)), _p(order, C.c_int32))

    def pt_serial(self, betas, ptswapever, neq, nmess, irinit, iconf, start, axis):
        nrep = len(betas)
        b = np.ascontiguousarray(betas, np.float64)
        sums = np.empty((nrep, NSUM))
        att = np.zeros(max(nrep - 1, 1), np.int64)
        acc = np.zeros(max(nrep - 1, 1), np.int64)
        vb = C.c_int32()
        spins = np.empty((nrep, self.N), np.int8)
        rat = np.empty(nrep, np.int32)
        lib().or_pt_serial_ref(self.ref(), C.c_int32(nrep), _p(b, C.c_double),
                               C.c_int32(ptswapever), C.c_int32(neq), C.c_int32(nmess),
                               C.c_int32(irinit), C.c_int32(iconf), C.c_int32(start),
                               C.c_int32(axis), _p(sums, C.c_double), _p(att, C.c_int64),
                               _p(acc, C.c_int64), C.byref(vb), _p(spins, C.c_int8),
                               _p(rat, C.c_int32))
        return dict(sums=sums, attempts=att[:nrep - 1], accepts=acc[:nrep - 1],
                    visitboth=vb.value, spins=spins, rep_at_temp=rat)

    def local(self, s0, beta, neq, nmess, kiss_state):
        lists = [np.empty(nmess) for _ in range(5)]
        s_out = np.empty(self.N, np.int8)
        lib().or_local_ref(self.ref(), _p(np.ascontiguousarray(s0, np.int8), C.c_int8),
                           C.c_double(beta), C.c_int32(neq), C.c_int32(nmess),
                           _p(kiss_state, C.c_uint32), *[_p(a, C.c_double) for a in lists],
                           _p(s_out, C.c_int8))
        return lists, s_out

    def bench_pt(self, nthreads, betas, ptswapever, ncycles, irinit=1) -> float:
        b = np.ascontiguousarray(betas, np.float64)
        return lib().or_bench_pt_ref(self.ref(), C.c_int32(nthreads), C.c_int32(len(b)),
                                     _p(b, C.c_double), C.c_int32(ptswapever),
                                     C.c_int32(ncycles), C.c_int32(irinit))

    # device-engine replay --------------------------------------------------------------------
    def replay_sweeps(self, s, beta, seed, conf, rep, sweep0, nsweeps, flipcounts=None):
        return lib().or_replay_sweeps(self.ref(), _p(s, C.c_int8), C.c_double(beta),
                                      C.c_uint32(seed), C.c_uint32(conf), C.c_uint32(rep),
                                      C.c_uint32(sweep0), C.c_int32(nsweeps),
                                      None if flipcounts is None else _p(flipcounts, C.c_int32))

    def wolff_step(self, s, beta, seed, conf, rep, cycle):
        """The engine's Wolff update restated (FP64 form); modifies s, returns the cluster size."""
        return lib().or_wolff_step(self.ref(), _p(s, C.c_int8), C.c_double(beta),
                                   C.c_uint32(seed), C.c_uint32(conf), C.c_uint32(rep),
                                   C.c_uint32(cycle))

    def replay_measure(self, s):
        ints = np.empty(4, np.int64)
        acc = C.c_int64()
        obs = np.empty(5)
        lib().or_replay_measure(self.ref(), _p(s, C.c_int8), _p(ints, C.c_int64), C.byref(acc),
                                _p(obs, C.c_double))
        return ints, acc.value, obs

    def replay_pt(self, state, betas, ptswapever, ncycles, cycle0, seed, conf, measure, phase0,
                  flips=None):
        """Advance ``state`` (dict of numpy arrays, modified in place) by ncycles PT cycles;
        ``flips`` (nrep x N int32, by temperature slot) accumulates accepted flips per site."""
        nrep = len(betas)
        b = np.ascontiguousarray(betas, np.float64)
        obs = np.empty((nrep, 5))
        lib().or_replay_pt(self.ref(), C.c_int32(nrep), _p(b, C.c_double), C.c_int32(ptswapever),
                           C.c_int32(ncycles), C.c_uint32(cycle0), C.c_uint32(seed),
                           C.c_uint32(conf), C.c_int32(int(measure)), C.c_int32(phase0),
                           _p(state["spins"], C.c_int8), _p(state["rep_at_temp"], C.c_int32),
                           _p(state["temp_of_rep"], C.c_int32), _p(state["sums"], C.c_double),
                           _p(state["nmeas"], C.c_int64), _p(state["attempts"], C.c_int64),
                           _p(state["accepts"], C.c_int64), _p(state["visited"], C.c_uint8),
                           _p(obs, C.c_double), None if flips is None else _p(flips, C.c_int32))
        return obs


def bench_pt_multi(models, nthreads, betas, ptswapever, ncycles, irinit=1) -> float:
    """Wall seconds of ncycles PT cycles of one ladder per model (the reference restatement:
    sequential site order, KISS, FP64), the ladders spread round-robin over nthreads threads;
    initialisation is not timed."""
    b = np.ascontiguousarray(betas, np.float64)
    arr = (C.POINTER(Lat) * len(models))(*[C.pointer(m.lat) for m in models])
    return lib().or_bench_pt_multi(arr, C.c_int32(len(models)), C.c_int32(nthreads),
                                   C.c_int32(len(b)), _p(b, C.c_double), C.c_int32(ptswapever),
                                   C.c_int32(ncycles), C.c_int32(irinit))


def new_pt_state(spins):
    """PT bookkeeping in the engine's conventions (0-based maps, slot sums, counters)."""
    nrep = spins.shape[0]
    sums = np.zeros((nrep, NSUM))
    sums[:, 20] = np.inf
    return dict(spins=np.ascontiguousarray(spins, np.int8),
                rep_at_temp=np.arange(nrep, dtype=np.int32),
                temp_of_rep=np.arange(nrep, dtype=np.int32), sums=sums,
                nmeas=np.zeros(nrep, np.int64), attempts=np.zeros(max(nrep, 1), np.int64),
                accepts=np.zeros(max(nrep, 1), np.int64), visited=np.zeros(nrep, np.uint8))


def neighbors(L: int, H: int) -> np.ndarray:
    m = np.empty(10 * L * L * H, np.int32)
    lib().or_neighbors(C.c_int32(L), C.c_int32(H), _p(m, C.c_int32))
    return m


def setup_vacancies(seed, L, H, pp=0.0, pph=0.0, ppv=0.0, mode=0):
    N = L * L * H
    m = neighbors(L, H)
    occu = np.empty(N, np.int8)
    jh = np.empty(N, np.int8)
    jv = np.empty(N, np.int8)
    nimp = lib().or_setup_vacancies(C.c_int32(seed), C.c_int32(L), C.c_int32(H), C.c_double(pp),
                                    C.c_double(pph), C.c_double(ppv), C.c_int32(mode),
                                    _p(m, C.c_int32), _p(occu, C.c_int8), _p(jh, C.c_int8),
                                    _p(jv, C.c_int8))
    return occu, jh, jv, nimp


def init_spins(seed, L, H, start, axis=0):
    s = np.empty(L * L * H, np.int8)
    lib().or_init_spins(C.c_int32(seed), C.c_int32(L), C.c_int32(H), C.c_int32(start),
                        C.c_int32(axis), _p(s, C.c_int8))
    return s


def hot_spins_philox(L, H, seed, conf, rep):
    s = np.empty(L * L * H, np.int8)
    lib().or_hot_spins_philox(C.c_int32(L), C.c_int32(H), C.c_uint32(seed), C.c_uint32(conf),
                              C.c_uint32(rep), _p(s, C.c_int8))
    return s


def ladder(n, tmin, tmax, split=False, tmid=9.5, tfrac=0.7):
    t = np.empty(n)
    lib().or_ladder(C.c_int32(n), C.c_double(tmin), C.c_double(tmax), C.c_int32(int(split)),
                    C.c_double(tmid), C.c_double(tfrac), _p(t, C.c_double))
    return t


def kiss_state(seed: int) -> np.ndarray:
    st = np.empty(4, np.uint32)
    lib().or_kiss_init(_p(st, C.c_uint32), C.c_int32(seed))
    return st


# ----------------------------------------------------------------------------------------------
# make_corr_rand_3d through the reference's Ooura FFT (golden-vector generator)
# ----------------------------------------------------------------------------------------------
def ref_corr_rand_3d(n1, n2, n3, xi, seed, do_uniform=True, max_value=2.0) -> np.ndarray:
    """Returns x with x[k, j, i] = x(i, j, k) of the Fortran routine (flat = site order)."""
    out = np.empty(n1 * n2 * n3, np.float64)
    ref_lib().ref_make_corr_rand_3d(_p(out, C.c_double), C.c_int(n1), C.c_int(n2), C.c_int(n3),
                                    C.c_double(xi), C.c_int(seed), C.c_int(int(do_uniform)),
                                    C.c_double(max_value))
    return out.reshape(n3, n2, n1)


# ------------------------------------------------------------------------------------------------
# Measurement-time diagnostics of the reference, restated for the tests
# ------------------------------------------------------------------------------------------------
def locnem_terms(s, occu, m):
    """One call of Accumulate_local_nematic_average (J:1009-1025): the per-site additions to
    locspin_accum and locnem_accum for spins s (site order), occupancy occu, neighbour table m
    (m[k*N:(k+1)*N] = slot m(k+1))."""
    N = s.size
    s = s.astype(np.int64)
    o = occu.astype(np.int64)
    m1, m2, m3, m4 = (m[k * N:(k + 1) * N] for k in range(4))
    ln = s * s[m3] * o[m3] - s * s[m1] * o[m1] + s * s[m4] * o[m4] - s * s[m2] * o[m2]
    return np.where(o == 1, s, 0), np.where(o == 1, ln, 0)


def pt_histogram(energies, bins):
    """WRITEHIST of the PT measurement loop (J:1514-1523) for one temperature slot: the range is
    set from the first measured energy, every sample lands in bin 1 + int((e - min) / size),
    clamped to [1, bins].  Returns (counts[bins], min, size)."""
    counts = np.zeros(bins)
    lo = size = 0.0
    for e in energies:
        e = float(e)
        if size <= 0.0:
            lo = e - (abs(e) + 1.0)
            hi = e + (abs(e) + 1.0)
            size = (hi - lo) / bins
        k = 1 + int((e - lo) / size)
        k = max(1, min(bins, k))
        counts[k - 1] += 1.0
    return counts, lo, size


def local_histogram_ref(enlist, bins):
    """WRITEHIST of the LOCAL sampler's Process_data (J:2296-2352): range from the min and max of
    the whole list widened by half the span (or +-1e-6 when flat), bin NINT((e - min) / size),
    samples outside 1..bins dropped.  Returns (counts[bins], min, size)."""
    lo, hi = float(min(enlist)), float(max(enlist))
    if hi > lo:
        span = hi - lo
        lo -= 0.5 * span
        hi += 0.5 * span
    if hi <= lo:
        lo -= 1.0e-6
        hi += 1.0e-6
    size = (hi - lo) / bins
    counts = np.zeros(bins)
    for e in enlist:
        x = (float(e) - lo) / size
        k = int(np.floor(x + 0.5)) if x >= 0 else -int(np.floor(-x + 0.5))
        if 1 <= k <= bins:
            counts[k - 1] += 1.0
    return counts, lo, size


def results_ref(sums_list, nmeas_list, nocc_list, temps):
    """Write_files' columns restated from the reference (J:1542-1684 per configuration, the sums
    of Collect_data, the formulas of Write_files J:3210-3575) for slot sums in SUM_FIELDS order.
    Returns {file stem: list of rows}; per-configuration files list (iconf, slot) rows."""
    temps = np.asarray(temps, np.float64)
    beta = 1.0 / temps
    per = []
    for S, nm, nocc in zip(sums_list, nmeas_list, nocc_list):
        n = np.asarray(nm, np.float64)
        f = {k: S[:, i] / n for i, k in enumerate(SUM_FIELDS[:20])}
        absmag, mag2, mag4, en, en2 = f["absmag"], f["mag2"], f["mag4"], f["en"], f["en2"]
        strx, stry = f["strx_abs"], f["stry_abs"]
        q = dict(absmag=absmag, mag2=mag2, mag4=mag4, en=en, strx=strx, stry=stry,
                 strx2=f["strx2"], strx4=f["strx4"], stry2=f["stry2"], stry4=f["stry4"],
                 str2=f["str2"], str4=f["str4"], absstr=f["absstr"], nem=f["nem"],
                 nbar=f["nbar"], nbarabs=f["nbarabs"], nbar2=f["nbar2"], nbar4=f["nbar4"])

        def b4(x4, x2):
            return np.where(x2 > 0, 1.0 - x4 / np.where(x2 > 0, 3.0 * x2 ** 2, 1.0), 0.0)
        q["susc"] = (mag2 - absmag ** 2) * nocc * beta
        q["suscstr"] = (q["str2"] - q["absstr"] ** 2) * nocc * beta
        q["UL"] = b4(mag4, mag2)
        q["US"] = np.where(q["str2"] > 0, 2.0 - q["str4"] / np.where(q["str2"] > 0, q["str2"] ** 2, 1), 0)
        q["USX"], q["USY"], q["UBN"] = b4(q["strx4"], q["strx2"]), b4(q["stry4"], q["stry2"]), \
            b4(q["nbar4"], q["nbar2"])
        q["sph"] = (en2 - en ** 2) * nocc * beta ** 2
        q["logmag"] = np.log(np.where(absmag > 0, absmag, np.finfo(float).tiny))
        q["stripediff"] = strx ** 2 - stry ** 2
        q["besten"], q["finalen"] = S[:, 20], S[:, 21]
        per.append(q)
    nf = len(per)

    def mean(k):
        return sum(p[k] for p in per) / nf

    def err(k):
        return np.sqrt(sum(p[k] ** 2 for p in per) / nf - mean(k) ** 2) / np.sqrt(nf)

    def coex(x, y):
        d = x * x + y * y
        return np.where(d > 0, 4 * x * x * y * y / np.where(d > 0, d * d, 1), 0.0)
    out = {}
    out["cfen"] = np.column_stack([temps, mean("en"), err("en"), mean("sph"), err("sph")])
    out["cfma"] = np.column_stack([temps, mean("absmag"), sum(p["absmag"] ** 2 for p in per) / nf,
                                   err("absmag"), mean("susc"), err("susc"), mean("UL"), err("UL"),
                                   mean("logmag"), 1 - mean("mag4") / (3 * mean("mag2") ** 2)])
    nb = mean("nbar")
    mabs = sum(np.abs(p["nbar"]) for p in per) / nf
    mabserr = np.sqrt(np.maximum(0, sum((np.abs(p["nbar"]) - mabs) ** 2 for p in per) / nf)) / np.sqrt(nf)
    nabs = mean("nbarabs")
    nabserr = np.sqrt(np.maximum(0, sum((p["nbarabs"] - nabs) ** 2 for p in per) / nf)) / np.sqrt(nf)
    n2, n4 = mean("nbar2"), mean("nbar4")
    out["cfnm"] = np.column_stack([temps, nb, mabs, nabs,
                                   np.sqrt(np.maximum(0, sum(p["nbar"] ** 2 for p in per) / nf - nb ** 2)) / np.sqrt(nf),
                                   mabserr, nabserr, n2, n4,
                                   np.where(n2 > 0, 1 - n4 / (3 * n2 ** 2), 0), mean("UBN"), err("UBN")])
    cp = sum(p["strx"] * p["stry"] for p in per) / nf
    cp2 = sum((p["strx"] * p["stry"]) ** 2 for p in per) / nf
    ca = sum(coex(p["strx"], p["stry"]) for p in per) / nf
    ca2 = sum(coex(p["strx"], p["stry"]) ** 2 for p in per) / nf
    s2, s4 = mean("str2"), mean("str4")
    out["cfst"] = np.column_stack([temps, mean("absstr"), s2, s4, mean("nem"), 2 - s4 / s2 ** 2,
                                   mean("suscstr"), mean("US"), err("US"),
                                   np.sqrt(sum(p["absstr"] ** 2 for p in per) / nf - mean("absstr") ** 2) / np.sqrt(nf),
                                   err("suscstr"), mean("strx"), mean("strx2"), mean("strx4"),
                                   mean("USX"), err("USX"), mean("stry"), mean("stry2"),
                                   mean("stry4"), mean("USY"), err("USY"), cp,
                                   np.sqrt(cp2 - cp ** 2) / np.sqrt(nf), ca,
                                   np.sqrt(ca2 - ca ** 2) / np.sqrt(nf)])
    out["cfxy"] = [[k + 1, temps[t], p["strx"][t], p["stry"][t], p["absstr"][t],
                    p["stripediff"][t], p["besten"][t], p["finalen"][t],
                    p["strx"][t] * p["stry"][t], float(coex(p["strx"][t], p["stry"][t]))]
                   for k, p in enumerate(per) for t in range(len(temps))]
    out["cfnd"] = [[k + 1, temps[t], p["nbar"][t], p["nbarabs"][t], p["nbar2"][t],
                    p["nbar4"][t], p["UBN"][t]] for k, p in enumerate(per) for t in range(len(temps))]
    return out
