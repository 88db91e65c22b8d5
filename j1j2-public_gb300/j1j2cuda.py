"""Python host side of libj1j2cuda (ctypes over the C ABI in include/j1j2c.h).

Mirrors the parts of sim/J1J2_6tv.f90 that sit around the GPU hot path: the run parameters
(J:43-96), the PT SERIAL driver (Initialize_pt_state J:1218-1247, Pt_equilibration_loop
J:1250-1279, Pt_measurement_loop J:1341-1684) and the LOCAL sampler (J:2122-2474), with the
sweeps, swaps and running sums executed by the CUDA engine.  There is no CPU fallback: every
call goes through libj1j2cuda.so and fails loudly when it cannot be loaded.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libj1j2cuda.so")

OK, EINVAL, ECUDA, ETIMEOUT, ENOMEM, ESTATE = 0, -1, -2, -3, -4, -5
FP64_PLAIN, FP32_BATCHED = 0, 1
START_HOT, START_FER, START_STR = 0, 1, 2
AXIS_X, AXIS_Y = 0, 1
FLAG_NO_GRAPH, FLAG_PROFILE, FLAG_GENERIC, FLAG_NO_FIXED, FLAG_GLOBAL = 1, 2, 4, 8, 16
FLAG_WOLFF = 32
FLAG_CLUSTER = 64
FLAG_WOLFF_CS2, FLAG_WOLFF_CS4 = 128, 256  # Wolff growth over 2 / 4 CTAs per lattice (testing)
FLAG_STREAM = 512  # streaming form of the shape-specialised kernels (testing)
FLAG_WOLFF_SPLIT = 1024  # Wolff + sweeps of cold and hot slots on two streams (HBM form; testing)
FLAG_WOLFF_BITS = 2048  # Wolff growth from bond activations decided beforehand (testing)
FLAG_PAIRS = 4096  # two replicas of one configuration per CTA in the shape-specialised kernels
FLAG_MULTI = 8192  # every lattice-shape group in one persistent launch (testing)
FLAG_COOP = 16384  # small batches: a cycle's colour phases in one cooperative launch (testing)
FLAG_REPLICA = 32768  # small batches: the lattice replicated in every CTA of a cluster (testing)
FLAG_WOLFF_ASYNC = 65536  # one-CTA Wolff growths without breadth-first levels (testing)

SUM_FIELDS = ("mag", "absmag", "mag2", "mag4", "en", "en2", "strx_abs", "stry_abs", "strx2",
              "strx4", "stry2", "stry4", "str2", "str4", "absstr", "nem", "nbar", "nbarabs",
              "nbar2", "nbar4", "best_en", "final_en")

EXPORTS = ("j1j2c_create", "j1j2c_create_multi", "j1j2c_conf_shape", "j1j2c_destroy", "j1j2c_last_error", "j1j2c_set_stream",
           "j1j2c_set_disorder", "j1j2c_set_ladder", "j1j2c_init_spins",
           "j1j2c_reset_measurements", "j1j2c_run", "j1j2c_enqueue", "j1j2c_sync",
           "j1j2c_metro_sweep_fp64", "j1j2c_audit_fp32",
           "j1j2c_get_slot_sums", "j1j2c_get_pt_stats", "j1j2c_get_maps", "j1j2c_get_spins",
           "j1j2c_get_observables", "j1j2c_get_profile", "j1j2c_get_config",
           "j1j2c_corr_rand_3d", "j1j2c_setup_vacancies", "j1j2c_kiss_spins", "j1j2c_ladder",
           "j1j2c_version", "j1j2c_wolff", "j1j2c_get_cluster_sizes", "j1j2c_enumerate_exact",
           "j1j2c_set_diagnostics", "j1j2c_get_locnem", "j1j2c_get_histogram", "j1j2c_get_trace",
           "j1j2c_get_flip_counts", "j1j2c_state_size", "j1j2c_save_state", "j1j2c_load_state",
           "j1j2c_get_diagnostics", "j1j2c_get_occupied", "j1j2c_corr_rand_3d_gpu",
           "j1j2c_results_create", "j1j2c_results_add_conf", "j1j2c_results_write",
           "j1j2c_results_destroy", "j1j2c_set_retry_budget", "j1j2c_inject_fault",
           "j1j2c_enumerate_exact_noalloc")

ENUM_FIELDS = ("lnZ", "e", "e2", "absm", "m2", "m4", "abssx", "sx2", "abssy", "sy2", "nbar",
               "nbar2")


class J1J2CError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libj1j2cuda error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("L", C.c_int32), ("H", C.c_int32), ("J1h", C.c_double), ("J1v", C.c_double),
                ("J2", C.c_double), ("J3", C.c_double), ("nconf", C.c_int32),
                ("nreplica", C.c_int32), ("ptswapever", C.c_int32), ("precision", C.c_int32),
                ("seed", C.c_uint32), ("conf_base", C.c_uint32), ("device", C.c_int32),
                ("flags", C.c_uint32), ("block_threads", C.c_int32)]


class SlotSums(C.Structure):
    _fields_ = [(f, C.c_double) for f in SUM_FIELDS] + [("nmeasure", C.c_int64)]


class RunInfo(C.Structure):
    _fields_ = [("L", C.c_int32), ("H", C.c_int32)] + \
        [(f, C.c_double) for f in ("J1", "deltaJ1", "J2", "J3", "phi", "xi", "pp")] + \
        [(f, C.c_char_p) for f in ("impmode", "start", "straxis", "samplermode", "updateorder",
                                    "tempprotocol", "ptstartmode", "ptladdermode")] + \
        [(f, C.c_int32) for f in ("nreplica", "ptswapever", "ptmeasindex", "nconf", "neq",
                                   "nmess", "irinit")] + \
        [("tladdermid", C.c_double), ("tladderfrac", C.c_double)] + \
        [(f, C.c_int32) for f in ("bins", "write_strip", "write_numflips", "write_phitable")]


class Diagnostics(C.Structure):
    _fields_ = [("locnem_slot", C.c_int32), ("hist_bins", C.c_int32),
                ("trace_cycles", C.c_int32), ("flip_counts", C.c_int32)]


_lib = None


def lib():
    """Load libj1j2cuda.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run j1j2-public_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name in EXPORTS:
            getattr(L, name)
        L.j1j2c_last_error.restype = C.c_char_p
        L.j1j2c_last_error.argtypes = [C.c_void_p]
        L.j1j2c_version.restype = C.c_char_p
        L.j1j2c_destroy.restype = None
        L.j1j2c_results_destroy.restype = None
        L.j1j2c_results_destroy.argtypes = [C.c_void_p]
        L.j1j2c_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _check(ctx, rc):
    if rc < 0:
        msg = lib().j1j2c_last_error(ctx)
        raise J1J2CError(rc, msg.decode() if msg else "")
    return rc


# ------------------------------------------------------------------------------------------------
# host helpers (no GPU)
# ------------------------------------------------------------------------------------------------
def corr_rand_3d(n1, n2, n3, xi, seed, do_uniform=True, max_value=2.0,
                 gpu=False) -> np.ndarray:
    """make_corr_rand_3d (CR:191-386); returns x[k, j, i] = x(i, j, k), i.e. site order.
    gpu=True runs the transforms on the current GPU (cuFFT)."""
    out = np.empty(n1 * n2 * n3, np.float64)
    fn = lib().j1j2c_corr_rand_3d_gpu if gpu else lib().j1j2c_corr_rand_3d
    _check(None, fn(C.c_int32(n1), C.c_int32(n2), C.c_int32(n3), C.c_double(xi),
                    C.c_int32(seed), C.c_int32(int(do_uniform)), C.c_double(max_value),
                    _p(out, C.c_double)))
    return out.reshape(n3, n2, n1)


def setup_vacancies(seed, L, H, pp=0.0, pph=0.0, ppv=0.0, mode=0):
    """Setup_vacancies (J:1111-1165) after kissinit(seed): (occu, jh, jv, nimp)."""
    N = L * L * H
    occu, jh, jv = (np.empty(N, np.int8) for _ in range(3))
    nimp = _check(None, lib().j1j2c_setup_vacancies(
        C.c_int32(seed), C.c_int32(L), C.c_int32(H), C.c_double(pp), C.c_double(pph),
        C.c_double(ppv), C.c_int32(mode), _p(occu, C.c_int8), _p(jh, C.c_int8),
        _p(jv, C.c_int8)))
    return occu, jh, jv, nimp


def kiss_spins(seed, L, H, start, axis=AXIS_X) -> np.ndarray:
    """Initialize_spin_array (J:1179-1209) after kissinit(seed)."""
    s = np.empty(L * L * H, np.int8)
    _check(None, lib().j1j2c_kiss_spins(C.c_int32(seed), C.c_int32(L), C.c_int32(H),
                                        C.c_int32(start), C.c_int32(axis), _p(s, C.c_int8)))
    return s


def ladder(n, tmin, tmax, split=False, tmid=9.5, tfrac=0.7) -> np.ndarray:
    """Setup_temperature_ladder (J:928-962, PT branch)."""
    t = np.empty(n)
    _check(None, lib().j1j2c_ladder(C.c_int32(n), C.c_double(tmin), C.c_double(tmax),
                                    C.c_int32(int(split)), C.c_double(tmid), C.c_double(tfrac),
                                    _p(t, C.c_double)))
    return t


def enumerate_exact(L, H, p, betas, occu=None, jh=None, jv=None, J1h=1.0, J1v=1.0, J2=-1.0,
                    J3=1.0) -> np.ndarray:
    """Exact averages over all 2^N states (N <= 32) on the GPU: (len(betas), 12) in ENUM_FIELDS
    order (ln Z, then per-site <e>, <e^2>, <|m|>, <m^2>, <m^4>, <|sx|>, <sx^2>, <|sy|>, <sy^2>,
    <nbar>, <nbar^2>)."""
    p = np.ascontiguousarray(p, np.float64).reshape(-1)
    b = np.ascontiguousarray(betas, np.float64).reshape(-1)
    out = np.empty((b.size, 12))
    arrs = [None if a is None else np.ascontiguousarray(a, np.int8).reshape(-1)
            for a in (occu, jh, jv)]
    ptrs = [None if a is None else _p(a, C.c_int8) for a in arrs]
    _check(None, lib().j1j2c_enumerate_exact(C.c_int32(L), C.c_int32(H), C.c_double(J1h),
                                             C.c_double(J1v), C.c_double(J2), C.c_double(J3),
                                             _p(p, C.c_double), *ptrs, C.c_int32(b.size),
                                             _p(b, C.c_double), _p(out, C.c_double)))
    return out


INJECT_NONE, INJECT_ALLOC, INJECT_LAUNCH = 0, 1, 2


def inject_fault(kind):
    """One-shot failure of the next device allocation (INJECT_ALLOC) or PT-cycle launch
    (INJECT_LAUNCH) of any engine context, reported without touching the device (tests)."""
    _check(None, lib().j1j2c_inject_fault(C.c_int32(kind)))


def disorder(L, H, seed, phi=2.0, xi=3.0, map_uniform=True, gpu=False) -> np.ndarray:
    """Setup_phi_table (J:590-633): p(site) for disorder seed IRINIT + iconf - 1."""
    return corr_rand_3d(L, L, H, xi, seed, map_uniform, phi, gpu).reshape(-1)


# ------------------------------------------------------------------------------------------------
# engine context
# ------------------------------------------------------------------------------------------------
class Engine:
    """One libj1j2cuda context: nconf disorder configurations x nreplica ladder replicas, or
    several lattice-shape groups (``groups=[(L, H, nconf, nreplica), ...]``) in one batch."""

    def __init__(self, L=None, H=None, nconf=1, nreplica=1, ptswapever=5, precision=FP32_BATCHED,
                 seed=1, conf_base=0, J1h=1.0, J1v=1.0, J2=-1.0, J3=1.0, device=0, flags=0,
                 block_threads=0, groups=None):
        if groups is None:
            groups = [(L, L if H is None else H, nconf, nreplica, block_threads)]
        groups = [tuple(g) + (block_threads,) * (5 - len(g)) for g in groups]
        self.ptswapever, self.precision = int(ptswapever), precision
        arr = (Params * len(groups))()
        for k, (gL, gH, gn, gr, gbt) in enumerate(groups):
            arr[k] = Params(gL, gH, J1h, J1v, J2, J3, gn, gr, self.ptswapever, precision, seed,
                            conf_base, device, flags, gbt)
        self.params = arr
        self._ctx = C.c_void_p()
        _check(None, lib().j1j2c_create_multi(C.byref(self._ctx), arr, C.c_int32(len(groups))))
        self.shapes = []  # per conf: (L, H, nreplica)
        for gL, gH, gn, gr, _ in groups:
            self.shapes += [(int(gL), int(gH), int(gr))] * int(gn)
        self.nconf = len(self.shapes)
        self.L, self.H, _, _, _ = (int(v) for v in groups[0])
        self.nrep = int(groups[0][3])
        self.N = self.L * self.L * self.H
        self.rbase = np.cumsum([0] + [s[2] for s in self.shapes])
        self.nentries = int(self.rbase[-1])
        self.nocc = np.array([s[0] * s[0] * s[1] for s in self.shapes], np.int64)
        self.diag = Diagnostics(-1, 0, 0, 0)

    def _shape(self, conf):
        if not 0 <= conf < self.nconf:
            raise J1J2CError(EINVAL, f"conf {conf} out of range")
        return self.shapes[conf]

    def n_of(self, conf):
        L, H, _ = self._shape(conf)
        return L * L * H

    def nrep_of(self, conf):
        return self._shape(conf)[2]

    # life cycle --------------------------------------------------------------------------------
    def close(self):
        if self._ctx:
            lib().j1j2c_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def _ck(self, rc):
        return _check(self._ctx, rc)

    def set_stream(self, stream_ptr):
        self._ck(lib().j1j2c_set_stream(self._ctx, C.c_void_p(stream_ptr)))

    # inputs ------------------------------------------------------------------------------------
    def set_disorder(self, conf, p, occu=None, jh=None, jv=None):
        p = np.ascontiguousarray(p, np.float64).reshape(-1)
        assert p.size == self.n_of(conf)
        arrs = [None if a is None else np.ascontiguousarray(a, np.int8).reshape(-1)
                for a in (occu, jh, jv)]
        ptrs = [None if a is None else _p(a, C.c_int8) for a in arrs]
        self._ck(lib().j1j2c_set_disorder(self._ctx, C.c_int32(conf), _p(p, C.c_double), *ptrs))
        self.nocc[conf] = p.size if arrs[0] is None else int((arrs[0] != 0).sum())

    def set_ladder(self, conf, beta):
        """beta of one conf (nrep), or of every conf when conf < 0 (nconf x nrep)."""
        b = np.ascontiguousarray(beta, np.float64)
        assert b.size == (self.nentries if conf < 0 else self.nrep_of(conf))
        self._ck(lib().j1j2c_set_ladder(self._ctx, C.c_int32(conf), _p(b, C.c_double)))

    def init_spins(self, conf, start=START_HOT, axis=AXIS_X, spins=None):
        if spins is None:
            self._ck(lib().j1j2c_init_spins(self._ctx, C.c_int32(conf), C.c_int32(start),
                                            C.c_int32(axis), None))
        else:
            s = np.ascontiguousarray(spins, np.int8).reshape(self.nrep_of(conf), self.n_of(conf))
            self._ck(lib().j1j2c_init_spins(self._ctx, C.c_int32(conf), C.c_int32(start),
                                            C.c_int32(axis), _p(s, C.c_int8)))

    def reset_measurements(self, conf=-1):
        self._ck(lib().j1j2c_reset_measurements(self._ctx, C.c_int32(conf)))

    # hot path ----------------------------------------------------------------------------------
    def run(self, ncycles, measure=True, restart_swap_phase=True):
        self._ck(lib().j1j2c_run(self._ctx, C.c_int32(ncycles), C.c_int32(int(measure)),
                                 C.c_int32(int(restart_swap_phase))))

    def enqueue(self, ncycles, measure=True, restart_swap_phase=True):
        """run() without waiting: the cycles are queued on the context's stream; sync() waits."""
        self._ck(lib().j1j2c_enqueue(self._ctx, C.c_int32(ncycles), C.c_int32(int(measure)),
                                     C.c_int32(int(restart_swap_phase))))

    def sync(self):
        self._ck(lib().j1j2c_sync(self._ctx))

    def metro_sweep_fp64(self, conf, rep, beta, sweep_index, nsweeps=1):
        out = [C.c_double() for _ in range(4)]
        self._ck(lib().j1j2c_metro_sweep_fp64(self._ctx, C.c_int32(conf), C.c_int32(rep),
                                              C.c_double(beta), C.c_uint32(sweep_index),
                                              C.c_int32(nsweeps), *[C.byref(o) for o in out]))
        return tuple(o.value for o in out)

    def set_retry_budget(self, tries):
        """Union-find attempts per bond before the labelling forms of the Wolff update give up
        (default 2^20; the call then raises ETIMEOUT and the context stays usable)."""
        self._ck(lib().j1j2c_set_retry_budget(self._ctx, C.c_int32(tries)))

    def wolff(self):
        """One Wolff update of every lattice; returns the flipped-cluster sizes per replica."""
        out = np.zeros(self.nentries, np.int64)
        self._ck(lib().j1j2c_wolff(self._ctx, _p(out, C.c_int64)))
        return out

    # diagnostics -------------------------------------------------------------------------------
    def set_diagnostics(self, locnem_slot=-1, hist_bins=0, trace_cycles=0, flip_counts=False):
        """WRITELOCNEM (slot = PTMEASINDEX - 1), WRITEHIST (BINS), per-cycle traces and
        WRITENUMFLIPS of the reference's measurement loop; everything off by default."""
        d = Diagnostics(int(locnem_slot), int(hist_bins), int(trace_cycles), int(bool(flip_counts)))
        self._ck(lib().j1j2c_set_diagnostics(self._ctx, C.byref(d)))
        self.diag = d

    def locnem(self, conf):
        """(locspin_accum, locnem_accum, locnem_samples) of one conf in site order (J:1009-1025)."""
        n = self.n_of(conf)
        ls, ln = np.empty(n), np.empty(n)
        ns = C.c_int64()
        self._ck(lib().j1j2c_get_locnem(self._ctx, C.c_int32(conf), _p(ls, C.c_double),
                                        _p(ln, C.c_double), C.byref(ns)))
        return ls, ln, ns.value

    def histogram(self, conf):
        """(counts[nrep, bins], emin[nrep], binsize[nrep]) of one conf (J:1514-1523)."""
        r = self.nrep_of(conf)
        counts = np.empty((r, self.diag.hist_bins))
        lo, bs = np.empty(r), np.empty(r)
        self._ck(lib().j1j2c_get_histogram(self._ctx, C.c_int32(conf), _p(counts, C.c_double),
                                           _p(lo, C.c_double), _p(bs, C.c_double)))
        return counts, lo, bs

    def trace(self, conf):
        """(obs[cycles, nrep, 5] by slot, temp_of_rep[cycles, nrep]) of the recorded cycles."""
        r, cap = self.nrep_of(conf), max(1, self.diag.trace_cycles)
        obs = np.empty((cap, r, 5))
        tor = np.empty((cap, r), np.int32)
        n = C.c_int64()
        self._ck(lib().j1j2c_get_trace(self._ctx, C.c_int32(conf), _p(obs, C.c_double),
                                       _p(tor, C.c_int32), C.byref(n)))
        return obs[:n.value], tor[:n.value]

    def flip_counts(self, conf):
        """confnumflips of one conf: nrep x N int32 by slot in site order, -1 at vacancies."""
        out = np.empty((self.nrep_of(conf), self.n_of(conf)), np.int32)
        self._ck(lib().j1j2c_get_flip_counts(self._ctx, C.c_int32(conf), _p(out, C.c_int32)))
        return out

    # checkpoint / resume -----------------------------------------------------------------------
    def save_state(self) -> np.ndarray:
        """The whole device state as a byte array (write it to a file to checkpoint)."""
        n = C.c_int64()
        self._ck(lib().j1j2c_state_size(self._ctx, C.byref(n)))
        buf = np.empty(n.value, np.uint8)
        self._ck(lib().j1j2c_save_state(self._ctx, _p(buf, C.c_uint8), C.c_int64(buf.size)))
        return buf

    def load_state(self, buf):
        """Resume from save_state()'s bytes (a context created with the same parameters)."""
        b = np.ascontiguousarray(np.frombuffer(buf, np.uint8) if isinstance(buf, (bytes, bytearray))
                                 else buf, np.uint8)
        self._ck(lib().j1j2c_load_state(self._ctx, _p(b, C.c_uint8), C.c_int64(b.size)))
        d = Diagnostics()
        self._ck(lib().j1j2c_get_diagnostics(self._ctx, C.byref(d)))
        self.diag = d
        n = C.c_int32()
        for k in range(self.nconf):
            self._ck(lib().j1j2c_get_occupied(self._ctx, C.c_int32(k), C.byref(n)))
            self.nocc[k] = n.value

    def cluster_sizes(self, conf=-1):
        out = np.zeros(self.nentries if conf < 0 else self.nrep_of(conf), np.int64)
        self._ck(lib().j1j2c_get_cluster_sizes(self._ctx, C.c_int32(conf), _p(out, C.c_int64)))
        return out

    def audit_fp32(self, nsweeps):
        att, mis = C.c_int64(0), C.c_int64(0)
        self._ck(lib().j1j2c_audit_fp32(self._ctx, C.c_int32(nsweeps), C.byref(att),
                                        C.byref(mis)))
        return att.value, mis.value

    # outputs -----------------------------------------------------------------------------------
    SLOT_DTYPE = np.dtype([("s", np.float64, 22), ("n", np.int64)])

    def slot_sums(self, conf, out=None):
        """(nrep, 22) running sums in SUM_FIELDS order and the (nrep,) measurement counts;
        conf < 0 returns every conf, (nconf*nrep, 22) and (nconf*nrep,).  out: a record array
        of SLOT_DTYPE to fill (e.g. in pinned memory); the result is then views into it."""
        n = self.nentries if conf < 0 else self.nrep_of(conf)
        raw = np.zeros(n, dtype=self.SLOT_DTYPE) if out is None else out
        assert raw.dtype == self.SLOT_DTYPE and raw.size == n and raw.flags.c_contiguous
        self._ck(lib().j1j2c_get_slot_sums(self._ctx, C.c_int32(conf),
                                           raw.ctypes.data_as(C.c_void_p)))
        if out is not None:
            return raw["s"], raw["n"]
        return raw["s"].copy(), raw["n"].copy()

    def pt_stats(self, conf):
        nrep = self.nrep_of(conf)
        n = max(nrep - 1, 1)
        att, acc = np.zeros(n, np.int64), np.zeros(n, np.int64)
        vb = C.c_int32()
        self._ck(lib().j1j2c_get_pt_stats(self._ctx, C.c_int32(conf), _p(att, C.c_int64),
                                          _p(acc, C.c_int64), C.byref(vb)))
        return att[:nrep - 1], acc[:nrep - 1], vb.value

    def maps(self, conf):
        nrep = self.nrep_of(conf)
        rat, tor = np.empty(nrep, np.int32), np.empty(nrep, np.int32)
        self._ck(lib().j1j2c_get_maps(self._ctx, C.c_int32(conf), _p(rat, C.c_int32),
                                      _p(tor, C.c_int32)))
        return rat, tor

    def spins(self, conf, rep):
        s = np.empty(self.n_of(conf), np.int8)
        self._ck(lib().j1j2c_get_spins(self._ctx, C.c_int32(conf), C.c_int32(rep),
                                       _p(s, C.c_int8)))
        return s

    def observables(self, conf, out=None):
        """{mag, en, strx, stry, nbar} of every replica after the last cycle; out: an array of
        that shape to fill (e.g. in pinned memory)."""
        shape = (self.nentries if conf < 0 else self.nrep_of(conf), 5)
        if out is None:
            out = np.empty(shape)
        assert out.shape == shape and out.dtype == np.float64 and out.flags.c_contiguous
        self._ck(lib().j1j2c_get_observables(self._ctx, C.c_int32(conf), _p(out, C.c_double)))
        return out

    def profile(self):
        ms, n, att = C.c_double(), C.c_int64(), C.c_int64()
        self._ck(lib().j1j2c_get_profile(self._ctx, C.byref(ms), C.byref(n), C.byref(att)))
        return ms.value, n.value, att.value

    def config(self):
        bt, spt, sm = C.c_int32(), C.c_int32(), C.c_int32()
        self._ck(lib().j1j2c_get_config(self._ctx, C.byref(bt), C.byref(spt), C.byref(sm)))
        return dict(block_threads=bt.value, sites_per_thread=spt.value, smem_bytes=sm.value)


# ------------------------------------------------------------------------------------------------
# PT driver around the engine (Pt_measurement_loop finalisation, J:1542-1684)
# ------------------------------------------------------------------------------------------------
@dataclass
class SlotResult:
    T: np.ndarray
    mag: np.ndarray
    absmag: np.ndarray
    mag2: np.ndarray
    mag4: np.ndarray
    en: np.ndarray
    en2: np.ndarray
    strx: np.ndarray
    stry: np.ndarray
    absstr: np.ndarray
    nem: np.ndarray
    nbar: np.ndarray
    nbarabs: np.ndarray
    nbar2: np.ndarray
    nbar4: np.ndarray
    susc: np.ndarray
    suscstr: np.ndarray
    UL: np.ndarray
    US: np.ndarray
    USX: np.ndarray
    USY: np.ndarray
    UBN: np.ndarray
    sph: np.ndarray
    stripediff: np.ndarray
    best_en: np.ndarray
    final_en: np.ndarray


def finalize_slots(sums, nmeas, beta, nocc) -> SlotResult:
    """Per-slot thermal averages and derived quantities of one conf (J:1542-1600)."""
    s = np.asarray(sums, np.float64)
    n = np.maximum(np.asarray(nmeas, np.float64), 1.0)
    avg = s[:, :20] / n[:, None]
    mag = np.abs(s[:, 0]) / n
    absmag, mag2, mag4, en, en2 = avg[:, 1], avg[:, 2], avg[:, 3], avg[:, 4], avg[:, 5]
    strx, stry, strx2, strx4, stry2, stry4 = (avg[:, k] for k in range(6, 12))
    str2, str4, absstr, nem = avg[:, 12], avg[:, 13], avg[:, 14], avg[:, 15]
    nbar, nbarabs, nbar2, nbar4 = avg[:, 16], avg[:, 17], avg[:, 18], avg[:, 19]
    beta = np.asarray(beta, np.float64)

    def binder(m4, m2, a=1.0, b=3.0):
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(m2 > 0, a - m4 / (b * m2 ** 2), 0.0)

    return SlotResult(
        T=1.0 / beta, mag=mag, absmag=absmag, mag2=mag2, mag4=mag4, en=en, en2=en2, strx=strx,
        stry=stry, absstr=absstr, nem=nem, nbar=nbar, nbarabs=nbarabs, nbar2=nbar2, nbar4=nbar4,
        susc=(mag2 - absmag ** 2) * nocc * beta, suscstr=(str2 - absstr ** 2) * nocc * beta,
        UL=binder(mag4, mag2), US=np.where(str2 > 0, 2.0 - str4 / np.where(str2 > 0, str2, 1) ** 2,
                                            0.0),
        USX=binder(strx4, strx2), USY=binder(stry4, stry2), UBN=binder(nbar4, nbar2),
        sph=(en2 - en ** 2) * nocc * beta ** 2, stripediff=strx ** 2 - stry ** 2,
        best_en=s[:, 20], final_en=s[:, 21])


def local_histogram(enlist, bins):
    """WRITEHIST of the LOCAL sampler (Process_data, J:2296-2352) from the measured per-site
    energies of one temperature: the range spans the list's min..max widened by half the span on
    either side (+-1e-6 when flat), a sample goes to bin NINT((e - min) / size) and samples
    outside 1..bins are dropped.  Returns (counts[bins], min, size)."""
    e = np.asarray(enlist, np.float64)
    lo, hi = float(e.min()), float(e.max())
    if hi > lo:
        span = hi - lo
        lo, hi = lo - 0.5 * span, hi + 0.5 * span
    if hi <= lo:
        lo, hi = lo - 1.0e-6, hi + 1.0e-6
    size = (hi - lo) / bins
    x = (e - lo) / size
    k = np.where(x >= 0, np.floor(x + 0.5), -np.floor(-x + 0.5)).astype(np.int64)  # NINT
    k = k[(k >= 1) & (k <= bins)]
    return np.bincount(k - 1, minlength=bins).astype(np.float64), lo, size


class Results:
    """Disorder averages of a run written in the reference's file formats (Collect_data,
    J:2917-3207, and Write_files, J:3210-3575): cfen, cfma, cfnm, cfst, cfnd, and cfhs / cfxy /
    cfnu / cfpt / cfph as enabled."""

    def __init__(self, L, H, temps, nconf, neq, nmess, irinit=1, J1=1.0, deltaJ1=0.0, J2=-1.0,
                 J3=1.0, phi=2.0, xi=3.0, pp=0.0, impmode="RAN", start="HOT", straxis="X",
                 samplermode="PT   ", updateorder="SEQ", tempprotocol="INDEP",
                 ptstartmode="COMMON", ptladdermode="LINEAR", ptswapever=5, ptmeasindex=1,
                 tladdermid=9.5, tladderfrac=0.7, bins=0, write_strip=True,
                 write_numflips=False, write_phitable=False):
        self.temps = np.ascontiguousarray(temps, np.float64)
        self._strings = [x.encode() for x in (impmode, start, straxis, samplermode, updateorder,
                                              tempprotocol, ptstartmode, ptladdermode)]
        info = RunInfo(L, H, J1, deltaJ1, J2, J3, phi, xi, pp, *self._strings,
                       self.temps.size, ptswapever, ptmeasindex, nconf, neq, nmess, irinit,
                       tladdermid, tladderfrac, bins, int(write_strip), int(write_numflips),
                       int(write_phitable))
        self.N = L * L * H
        self.bins = bins
        self._res = C.c_void_p()
        _check(None, lib().j1j2c_results_create(C.byref(self._res), C.byref(info),
                                                _p(self.temps, C.c_double)))

    def add_conf(self, sums, nocc, attempts=None, accepts=None, visited_both=0, hist=None,
                 hist_min=None, hist_bin=None, flips=None, p=None):
        """sums: SLOT_DTYPE records (nrep) or a (22-column sums, counts) pair."""
        if isinstance(sums, tuple):
            rec = np.zeros(len(sums[1]), Engine.SLOT_DTYPE)
            rec["s"], rec["n"] = sums
            sums = rec
        arrs = []

        def ptr(a, dt, ct):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            arrs.append(a)
            return _p(a, ct)
        _check(None, lib().j1j2c_results_add_conf(
            self._res, sums.ctypes.data_as(C.c_void_p), C.c_int32(int(nocc)),
            ptr(attempts, np.int64, C.c_int64), ptr(accepts, np.int64, C.c_int64),
            C.c_int32(int(visited_both)), ptr(hist, np.float64, C.c_double),
            ptr(hist_min, np.float64, C.c_double), ptr(hist_bin, np.float64, C.c_double),
            ptr(flips, np.int32, C.c_int32), ptr(p, np.float64, C.c_double)))

    def add_engine_conf(self, eng, conf, p=None):
        """Pull one configuration's results from an Engine (diagnostics as enabled there)."""
        raw = np.zeros(eng.nrep_of(conf), Engine.SLOT_DTYPE)
        eng.slot_sums(conf, out=raw)
        att, acc, vb = eng.pt_stats(conf)
        hist = hmin = hbin = flips = None
        if self.bins > 0 and eng.diag.hist_bins == self.bins:
            hist, hmin, hbin = eng.histogram(conf)
        if eng.diag.flip_counts:
            flips = eng.flip_counts(conf)
        self.add_conf(raw, eng.nocc[conf], att, acc, vb, hist, hmin, hbin, flips, p)

    def write(self, directory):
        os.makedirs(directory, exist_ok=True)
        _check(None, lib().j1j2c_results_write(self._res, os.fsencode(directory)))

    def close(self):
        if self._res:
            lib().j1j2c_results_destroy(self._res)
            self._res = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pt_run(L, betas, nconf=1, neq=100, nmess=100, ptswapever=5, irinit=1, start=START_HOT,
           axis=AXIS_X, phi=2.0, xi=3.0, pp=0.0, precision=FP32_BATCHED, H=None, engine=None):
    """PT SERIAL over nconf disorder configurations resident together on the GPU.

    Disorder seed of conf k is IRINIT + k (J:317, J:611); vacancies as Setup_vacancies.
    Returns (engine, [SlotResult per conf], [pt stats per conf])."""
    H = L if H is None else H
    nrep = len(betas)
    eng = engine or Engine(L, H, nconf=nconf, nreplica=nrep, ptswapever=ptswapever,
                           precision=precision, seed=irinit)
    for k in range(nconf):
        seed = irinit + k
        occu = None
        if pp > 0.0:
            occu, _, _, _ = setup_vacancies(seed, L, H, pp)
        eng.set_disorder(k, disorder(L, H, seed, phi, xi), occu)
        eng.set_ladder(k, betas)
        eng.init_spins(k, start, axis)
    eng.reset_measurements()
    eng.run(neq, measure=False, restart_swap_phase=True)
    eng.reset_measurements()
    eng.run(nmess, measure=True, restart_swap_phase=True)
    results, stats = [], []
    for k in range(nconf):
        sums, nm = eng.slot_sums(k)
        results.append(finalize_slots(sums, nm, betas, eng.nocc[k]))
        stats.append(eng.pt_stats(k))
    return eng, results, stats
