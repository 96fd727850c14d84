"""Batched Monte Carlo state and the Carlo.jl-style driver callbacks.

``Engine`` owns one libkvmc handle (a batch of walkers on one GPU).  ``MC``
mirrors the reference's ``MC`` plus its Carlo.jl callbacks
(src/MonteCarlo.jl:165-185, :435-441, :538-755): ``init_``, ``sweep_``,
``measure_``, ``register_evaluables``, ``write_checkpoint``,
``read_checkpoint_``.  One ``sweep_`` call makes ``proposals_per_sweep``
proposals per walker (1 by default, one reference ``sweep!`` call each).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import ArgumentError, SingularException
from .lattice import PI_LINK_IN, PI_LINK_INTER, DoubleKagome, Hamiltonian


class Engine:
    """A batch of walkers of one model on one GPU (a kvmc handle)."""

    def __init__(self, ham: Hamiltonian, n_walkers=1, precision="plain", accept="reference",
                 refresh_interval=0, measure_interval=0, seed=0, device=0, delay_k=0, w_placement="auto"):
        self.ham = ham
        self.N = int(ham.U_up.shape[0])
        self.n_up = int(ham.U_up.shape[1])
        self.n_down = int(ham.U_down.shape[1])
        self.n_walkers = int(n_walkers)
        prec = {"plain": _lib.PLAIN_FP64, "mixed": _lib.MIXED_FP32}.get(precision, precision)
        acc = {"reference": _lib.ACCEPT_REFERENCE, "metropolis": _lib.ACCEPT_METROPOLIS}.get(accept, accept)
        self.mixed = prec == _lib.MIXED_FP32
        self.n_params = 0
        self._bonds = _lib.as_c(np.asarray(ham.nn, dtype=np.int32).reshape(-1), np.int32)
        # complex orbitals (B != 0) make a complex handle: W, ratios complex
        self.complex = bool(np.iscomplexobj(ham.U_up) or np.iscomplexobj(ham.U_down))
        self._Uu = np.asfortranarray(np.real(ham.U_up), dtype=np.float64)
        self._Ud = np.asfortranarray(np.real(ham.U_down), dtype=np.float64)
        md = _lib.ModelDesc()
        md.n_sites, md.n_up, md.n_down = self.N, self.n_up, self.n_down
        md.n_bonds = len(ham.nn)
        md.bonds = self._bonds.ctypes.data_as(C.POINTER(C.c_int32))
        md.U_up = self._Uu.ctypes.data_as(C.POINTER(C.c_double))
        md.U_down = self._Ud.ctypes.data_as(C.POINTER(C.c_double))
        if self.complex:
            self._Uui = np.asfortranarray(np.imag(ham.U_up), dtype=np.float64)
            self._Udi = np.asfortranarray(np.imag(ham.U_down), dtype=np.float64)
            md.U_up_imag = self._Uui.ctypes.data_as(C.POINTER(C.c_double))
            md.U_down_imag = self._Udi.ctypes.data_as(C.POINTER(C.c_double))
        bd = _lib.BatchDesc()
        bd.n_walkers, bd.precision, bd.accept_rule = self.n_walkers, prec, acc
        bd.refresh_interval, bd.measure_interval = int(refresh_interval), int(measure_interval)
        bd.delay_k, bd.device, bd.seed = int(delay_k), int(device), int(seed) & 0xFFFFFFFFFFFFFFFF
        bd.w_placement = {"auto": 0, "chip": 1, "hbm": 2}.get(w_placement, w_placement)
        self._lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self._lib.kvmc_create(C.byref(md), C.byref(bd), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._lib.kvmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _lib.check(rc, self.h)

    # --- state ---------------------------------------------------------------
    def init(self, kappa_up=None, kappa_down=None):
        att = np.zeros(self.n_walkers, dtype=np.int32)
        if kappa_up is None:
            self._check(self._lib.kvmc_init(self.h, None, None, _lib.ptr(att)))
        else:
            ku = _lib.as_c(np.broadcast_to(kappa_up, (self.n_walkers, self.N)), np.int32)
            kd = _lib.as_c(np.broadcast_to(kappa_down, (self.n_walkers, self.N)), np.int32)
            self._check(self._lib.kvmc_init(self.h, _lib.ptr(ku), _lib.ptr(kd), _lib.ptr(att)))
        return att

    def get_state(self):
        ku = np.empty((self.n_walkers, self.N), dtype=np.int32)
        kd = np.empty_like(ku)
        ct = np.empty(self.n_walkers, dtype=np.int64)
        self._check(self._lib.kvmc_get_state(self.h, _lib.ptr(ku), _lib.ptr(kd), _lib.ptr(ct)))
        return ku, kd, ct

    def set_state(self, kappa_up, kappa_down, counters=None):
        ku = _lib.as_c(np.broadcast_to(kappa_up, (self.n_walkers, self.N)), np.int32)
        kd = _lib.as_c(np.broadcast_to(kappa_down, (self.n_walkers, self.N)), np.int32)
        ct = None if counters is None else _lib.as_c(np.broadcast_to(counters, (self.n_walkers,)), np.int64)
        self._check(self._lib.kvmc_set_state(self.h, _lib.ptr(ku), _lib.ptr(kd), _lib.ptr(ct)))

    def get_w(self):
        dt = np.complex128 if self.complex else np.float64
        Wu = np.empty((self.n_walkers, self.N, self.n_up), dtype=dt)
        Wd = np.empty((self.n_walkers, self.N, self.n_down), dtype=dt)
        self._check(self._lib.kvmc_get_w(self.h, _lib.ptr(Wu), _lib.ptr(Wd)))
        return Wu, Wd

    # --- hot path ------------------------------------------------------------
    def sweep(self, proposals_per_walker: int) -> dict:
        st = _lib.SweepStats()
        self._check(self._lib.kvmc_sweep(self.h, int(proposals_per_walker), C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def advance(self, moves_per_walker: int) -> dict:
        """Every walker makes `moves_per_walker` more accepted moves."""
        st = _lib.SweepStats()
        self._check(self._lib.kvmc_advance(self.h, int(moves_per_walker), C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def measure(self) -> np.ndarray:
        out = np.empty(self.n_walkers)
        self._check(self._lib.kvmc_measure(self.h, _lib.ptr(out)))
        return out

    def refresh(self):
        self._check(self._lib.kvmc_refresh(self.h))

    def eval_ratios(self, moves) -> np.ndarray:
        mv = _lib.as_c(moves, np.int32)
        if mv.ndim == 2:
            mv = mv[None]
        mv = _lib.as_c(np.broadcast_to(mv, (self.n_walkers, mv.shape[1], 4)), np.int32)
        out = np.empty((self.n_walkers, mv.shape[1]), dtype=np.complex128 if self.complex else np.float64)
        self._check(self._lib.kvmc_eval_ratios(self.h, mv.shape[1], _lib.ptr(mv), _lib.ptr(out)))
        return out

    def apply_moves(self, moves):
        mv = _lib.as_c(np.broadcast_to(np.asarray(moves, dtype=np.int32), (self.n_walkers, 5)), np.int32)
        self._check(self._lib.kvmc_apply_moves(self.h, _lib.ptr(mv)))

    def walker_stats(self) -> dict:
        Wk = self.n_walkers
        se, se2 = np.empty(Wk), np.empty(Wk)
        nm, acc, prop = (np.empty(Wk, dtype=np.int64) for _ in range(3))
        status = np.empty(Wk, dtype=np.int32)
        self._check(self._lib.kvmc_walker_stats(self.h, _lib.ptr(se), _lib.ptr(se2), _lib.ptr(nm), _lib.ptr(acc),
                                                _lib.ptr(prop), _lib.ptr(status)))
        return dict(sum_e=se, sum_e2=se2, n_meas=nm, accepted=acc, proposals=prop, status=status)

    # --- adjoint gradient ------------------------------------------------------
    def set_log_derivatives(self, dU_up, dU_down):
        """dU_sigma: [P][N][n_sigma] orbital derivatives (complex or real)."""
        dU_up, dU_down = np.asarray(dU_up), np.asarray(dU_down)
        P = dU_up.shape[0]
        # [P][n][N] C order = P column-major N x n matrices
        def split(d):
            t = np.ascontiguousarray(np.transpose(d, (0, 2, 1)))
            return (np.ascontiguousarray(t.real, dtype=np.float64),
                    np.ascontiguousarray(t.imag, dtype=np.float64) if np.iscomplexobj(t) else None)
        ur, ui = split(dU_up)
        dr, di = split(dU_down)
        self._check(self._lib.kvmc_set_log_derivatives(self.h, P, _lib.ptr(ur), _lib.ptr(ui), _lib.ptr(dr),
                                                       _lib.ptr(di)))
        self.n_params = P

    def measure_grad(self, want=False):
        """One adjoint evaluation at every walker's configuration; with want=True
        returns (E_L complex [W], O complex [W][P])."""
        if not want:
            self._check(self._lib.kvmc_measure_grad(self.h, None, None))
            return None
        e = np.empty((self.n_walkers, 2))
        o = np.empty((self.n_walkers, self.n_params, 2))
        self._check(self._lib.kvmc_measure_grad(self.h, _lib.ptr(e), _lib.ptr(o)))
        return e[:, 0] + 1j * e[:, 1], o[..., 0] + 1j * o[..., 1]

    def grad_sums(self) -> np.ndarray:
        P = self.n_params
        out = np.empty((self.n_walkers, 3 + 4 * P + 2 * P * P))
        self._check(self._lib.kvmc_grad_sums(self.h, _lib.ptr(out)))
        return out

    def walker_logdet(self) -> np.ndarray:
        out = np.empty((self.n_walkers, 2))
        self._check(self._lib.kvmc_walker_logdet(self.h, _lib.ptr(out)))
        return out

    def walker_drift(self) -> np.ndarray:
        d = np.empty(self.n_walkers, dtype=np.float32)
        self._check(self._lib.kvmc_walker_drift(self.h, _lib.ptr(d)))
        return d

    def set_pipeline(self, on: bool = True):
        """Delayed form: scan for the next move while the last one's factor column is written."""
        self._check(self._lib.kvmc_set_tuning(self.h, 2, int(bool(on))))

    def set_refresh32(self, mode=True):
        """Periodic refresh by FP32 iterative refinement (FP64 fallback per
        walker): True / 1 = one thread per row, 2 or "tiled" = tiles of 32 rows
        per CTA (faster from about 200 orbitals per spin), 3 or "tc" = tiled
        with the refinement's residual on the tensor cores (exact bf16 digit
        products), False / 0 = FP64."""
        value = 2 if mode in (2, "tiled") else 3 if mode in (3, "tc") else int(bool(mode))
        self._check(self._lib.kvmc_set_tuning(self.h, 4, value))

    def set_cluster(self, ctas: int):
        """Mixed real form with rank-1 updates (delay_k 1): W split over a
        thread-block cluster of 2 or 4 CTAs per walker (0 = off)."""
        self._check(self._lib.kvmc_set_tuning(self.h, 10, int(ctas)))

    def set_drift_severe(self, factor: int):
        """One CTA per walker, delayed form: a drift past `factor` tolerances
        refreshes at once inside a call (0 = the default max(100 tol, 1e-2));
        milder drift waits for the end of the call."""
        self._check(self._lib.kvmc_set_tuning(self.h, 9, int(factor)))

    def set_tc_flush(self, on: bool = True):
        """W in HBM: rank-k flush on the tensor cores (tcgen05, 3xTF32)."""
        self._check(self._lib.kvmc_set_tuning(self.h, 3, int(bool(on))))

    def set_stream_threads(self, threads: int):
        """W in HBM: threads per walker's CTA (128 or 256)."""
        self._check(self._lib.kvmc_set_tuning(self.h, 1, int(threads)))

    def set_warp_walkers(self, walkers_per_cta: int):
        """0 = one CTA per walker; 1..14 = one warp per walker, this many per CTA
        (W's non-trivial rows indexed by labels; mixed real form, delay_k >= 4)."""
        self._check(self._lib.kvmc_set_tuning(self.h, 5, int(walkers_per_cta)))

    def set_accuracy_guard(self, hi: int, lo: int):
        """One-warp sweep: refresh a walker when its moves' |W| entries, after
        exceeding `hi` since its last refresh, are all below `lo` (0 = off); the
        refresh waits for the end of the call or segment when that is nearer
        than the refresh interval."""
        self._check(self._lib.kvmc_set_tuning(self.h, 6, int(hi)))
        self._check(self._lib.kvmc_set_tuning(self.h, 7, int(lo)))

    def set_segment(self, moves: int):
        """One-warp mode: advance in segments of this many accepted moves (0 = whole call)."""
        self._check(self._lib.kvmc_set_tuning(self.h, 8, int(moves)))

    def set_drift_tolerance(self, tol: float):
        self._check(self._lib.kvmc_set_drift_tolerance(self.h, float(tol)))

    def reset_stats(self):
        self._check(self._lib.kvmc_reset_stats(self.h))

    def enable_timing(self, on=True):
        self._check(self._lib.kvmc_enable_timing(self.h, int(bool(on))))

    def config(self) -> dict:
        r, m, k, on = (C.c_int32() for _ in range(4))
        self._check(self._lib.kvmc_get_config(self.h, C.byref(r), C.byref(m), C.byref(k), C.byref(on)))
        return dict(refresh_interval=r.value, measure_interval=m.value, delay_k=k.value, w_on_chip=bool(on.value))

    def region_start(self):
        self._check(self._lib.kvmc_region_timer(self.h, 1, None))

    def region_stop(self) -> float:
        ms = C.c_double()
        self._check(self._lib.kvmc_region_timer(self.h, 0, C.byref(ms)))
        return ms.value

    def kernel_time(self, kind: int):
        ms, n = C.c_double(), C.c_int64()
        self._check(self._lib.kvmc_kernel_time(self.h, int(kind), C.byref(ms), C.byref(n)))
        return ms.value, n.value


class Group:
    """Several engines (typically one per lattice size) advanced together by
    one captured CUDA graph (kvmc_group_*): each engine keeps its own
    delayed-update depth and refresh interval, and their launches run
    concurrently on the GPU."""

    def __init__(self, engines):
        self.engines = list(engines)
        self._lib = _lib.load()
        arr = (C.c_void_p * len(self.engines))(*[e.h.value if isinstance(e.h, C.c_void_p) else e.h
                                                 for e in self.engines])
        g = C.c_void_p()
        _lib.check(self._lib.kvmc_group_create(arr, len(self.engines), C.byref(g)))
        self.g = g

    def _check(self, rc):
        if rc != _lib.KVMC_OK:
            buf = C.create_string_buffer(1024)
            self._lib.kvmc_group_last_error(self.g, buf, len(buf))
            raise _lib._ERRORS.get(rc, _lib.DeviceError)(rc, buf.value.decode(errors="replace"))

    def advance(self, moves_per_walker: int):
        """Returns (per-engine stats, device ms of the graph launches)."""
        st = (_lib.SweepStats * len(self.engines))()
        ms = C.c_double()
        self._check(self._lib.kvmc_group_advance(self.g, int(moves_per_walker), st, C.byref(ms)))
        return [{k: getattr(s, k) for k, _ in s._fields_} for s in st], ms.value

    def close(self):
        if getattr(self, "g", None):
            self._lib.kvmc_group_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Carlo.jl-style plugin surface
# ---------------------------------------------------------------------------


@dataclass
class MCContext:
    """The part of Carlo.MCContext the callbacks use: a sweep counter and the measurement sink."""
    sweeps: int = 0
    thermalization: int = 0
    observables: dict = field(default_factory=dict)

    def measure(self, name, value):
        self.observables.setdefault(name, []).append(value)


class Evaluator:
    """The part of Carlo.Evaluator used by register_evaluables."""

    def __init__(self):
        self.evaluables = {}

    def evaluate(self, name, inputs, fn):
        self.evaluables[name] = (tuple(inputs), fn)

    def run(self, observables):
        out = {}
        for name, (inputs, fn) in self.evaluables.items():
            args = [np.mean(observables[i]) for i in inputs]
            out[name] = fn(*args)
        return out


class MC:
    """Batched counterpart of the reference ``MC`` (src/MonteCarlo.jl:17-28, :165-185).

    params: the reference keys (:n1, :n2, :PBC, :antiPBC, :lattice, :B,
    :N_up, :N_down, :link_in, :link_inter) as plain string keys, plus
    ``walkers``, ``precision`` ("plain" | "mixed"), ``accept``
    ("reference" | "metropolis"), ``refresh_interval``,
    ``measure_interval``, ``proposals_per_sweep``, ``seed``, ``device``,
    ``init`` ("qr" | "random"; default "qr" for one walker, else "random"),
    ``tuned`` (True: the mixed form with the autotuner's settings for this
    model and batch size from the shipped GB300 table, when it has them).
    """

    def __init__(self, params: dict):
        n1, n2 = params["n1"], params["n2"]
        lat_type = params.get("lattice", DoubleKagome)
        lat = lat_type(1.0, n1, n2, tuple(params["PBC"]), tuple(params.get("antiPBC", (False, False))))
        self.Ham = Hamiltonian.build(params["N_up"], params["N_down"], lat,
                                     link_in=params.get("link_in", PI_LINK_IN),
                                     link_inter=params.get("link_inter", PI_LINK_INTER),
                                     B=params.get("B", 0.0))
        self.params = dict(params)
        self.ns = n1 * n2 * 3
        self.walkers = int(params.get("walkers", 1))
        self.proposals_per_sweep = int(params.get("proposals_per_sweep", 1))
        choice = None
        if params.get("tuned", False):
            from . import autotune

            choice = autotune.lookup(self.Ham, self.walkers, params.get("accept", "reference"))
        if choice is not None:
            from . import autotune

            self.engine = autotune.make_engine(self.Ham, self.walkers, choice, accept=params.get("accept", "reference"),
                                               seed=params.get("seed", 0), device=params.get("device", 0))
        else:
            self.engine = Engine(self.Ham, self.walkers, params.get("precision", "plain"),
                                 params.get("accept", "reference"), params.get("refresh_interval", 0),
                                 params.get("measure_interval", 0), params.get("seed", 0), params.get("device", 0),
                                 params.get("delay_k", 0))
        self.n_occupied = min(self.Ham.N_up, self.Ham.N_down)
        self.last_stats = None   # the statistics of the last sweep_ call

    @property
    def kappa_up(self):
        return self.engine.get_state()[0]

    @property
    def kappa_down(self):
        return self.engine.get_state()[1]


def init_conf_qr(U_up, U_down, nsites, N_up):
    """Pivoted-QR start (src/MonteCarlo.jl:326-357), N_down = ns - N_up as at :339."""
    import scipy.linalg as sla
    _, _, p_up = sla.qr(np.asarray(U_up).T, mode="economic", pivoting=True)
    sites_up = [int(p) for p in p_up[:N_up]]
    ku = np.zeros(nsites, dtype=np.int32)
    ku[sites_up] = np.arange(1, N_up + 1)
    kd = np.zeros(nsites, dtype=np.int32)
    N_down = nsites - N_up
    if N_down > 0:
        avail = np.array([s for s in range(nsites) if s not in set(sites_up)])
        _, _, p_dn = sla.qr(np.asarray(U_down)[avail].T, mode="economic", pivoting=True)
        kd[avail[p_dn[:N_down]]] = np.arange(1, N_down + 1)
    return ku, kd


def init_(mc: MC, ctx: MCContext, params: dict):
    """Carlo.init! (src/MonteCarlo.jl:435-441, :382-410)."""
    mode = params.get("init", "qr" if mc.walkers == 1 else "random")
    if mode == "qr":
        ku, kd = init_conf_qr(mc.Ham.U_up, mc.Ham.U_down, mc.ns, params["N_up"])
        try:
            mc.engine.init(ku, kd)
        except SingularException as e:
            raise RuntimeError("QR-based configuration is singular. The Hamiltonian may be rank-deficient.") from e
    else:
        mc.engine.init()


def sweep_(mc: MC, ctx: MCContext):
    """Carlo.sweep! (src/MonteCarlo.jl:538-607): proposals_per_sweep proposals per walker.

    Records the batch acceptance fraction as ``acc`` (the reference records
    0.0 / 1.0 per call, :548-589)."""
    st = mc.engine.sweep(mc.proposals_per_sweep)
    mc.last_stats = st
    ctx.measure("acc", st["accepted"] / max(st["proposals"], 1))


def measure_(mc: MC, ctx: MCContext):
    """Carlo.measure! (src/MonteCarlo.jl:628-634): batch mean of the local energy.

    With a fused sweep (proposals_per_sweep of at least min(N_up, N_down)),
    the mean of the samples the last sweep_ took inside the library at the
    reference's cadence; otherwise a measurement of the current state when
    ctx.sweeps * proposals_per_sweep is a multiple of min(N_up, N_down)."""
    st = mc.last_stats
    if st is not None and st["measurements"] > 0:
        ctx.measure("OL", st["sum_energy"] / st["measurements"])
    elif (ctx.sweeps * mc.proposals_per_sweep) % mc.n_occupied == 0:
        ctx.measure("OL", float(np.mean(mc.engine.measure())))


def register_evaluables(cls, evaluator: Evaluator, params: dict):
    """Carlo.register_evaluables (src/MonteCarlo.jl:675-687): energy = OL / ns."""
    nsites = params["n1"] * params["n2"] * 3
    evaluator.evaluate("energy", ("OL",), lambda OL: OL / nsites)


def write_checkpoint(mc: MC, out):
    """Carlo.write_checkpoint (src/MonteCarlo.jl:715-719): kappa per walker, plus the
    per-walker position in the proposal stream.  `out` is any mapping (an
    h5py group works)."""
    ku, kd, ct = mc.engine.get_state()
    out["kappa_up"] = ku.astype(np.int64)
    out["kappa_down"] = kd.astype(np.int64)
    out["counters"] = ct


def read_checkpoint_(mc: MC, inp):
    """Carlo.read_checkpoint! (src/MonteCarlo.jl:751-755).  Unlike the reference, W is
    rebuilt from the restored configuration straight away."""
    ku = np.asarray(inp["kappa_up"])
    kd = np.asarray(inp["kappa_down"])
    ct = np.asarray(inp["counters"]) if "counters" in inp else None
    mc.engine.set_state(ku, kd, ct)
