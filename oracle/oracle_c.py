"""ctypes front end of the C oracle (kvmc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "kvmc_oracle.c"


def build(force=False):
    """Compiles the real and the complex-double oracle (gcc, no GPU)."""
    BUILD.mkdir(exist_ok=True)
    outs = {}
    for kind, flags in (("real", []), ("cplx", ["-DKVO_COMPLEX"])):
        out = BUILD / f"libkvmc_oracle_{kind}.so"
        if force or not out.exists() or out.stat().st_mtime < SRC.stat().st_mtime:
            cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", *flags, str(SRC), "-o", str(out), "-lm", "-lpthread"]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if r.returncode != 0:
                raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout.decode()}")
        outs[kind] = out
    return outs


class Model(C.Structure):
    _fields_ = [("n_sites", C.c_int32), ("n_up", C.c_int32), ("n_down", C.c_int32), ("n_bonds", C.c_int32),
                ("bonds", C.c_void_p), ("U_up", C.c_void_p), ("U_down", C.c_void_p)]


class Chain(C.Structure):
    _fields_ = [("kappa_up", C.c_void_p), ("kappa_down", C.c_void_p), ("W_up", C.c_void_p), ("W_down", C.c_void_p),
                ("t", C.c_int64), ("accepted", C.c_int64), ("sum_e", C.c_double), ("sum_e2", C.c_double),
                ("n_meas", C.c_int64), ("status", C.c_int32)]


_libs = {}


def lib(kind="real"):
    if kind not in _libs:
        path = build()[kind]
        L = C.CDLL(str(path))
        L.kvo_refresh.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        L.kvo_refresh.restype = C.c_int
        L.kvo_update_W.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.kvo_local_energy.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_int]
        L.kvo_local_energy.restype = C.c_double
        L.kvo_run_chain.argtypes = [C.POINTER(Model), C.POINTER(Chain), C.c_uint64, C.c_int, C.c_int64, C.c_int,
                                    C.c_int, C.c_int, C.c_void_p]
        L.kvo_run_chain.restype = C.c_int
        L.kvo_run_chains.argtypes = [C.POINTER(Model), C.POINTER(Chain), C.c_int, C.c_uint64, C.c_int64, C.c_int,
                                     C.c_int, C.c_int, C.c_int]
        L.kvo_run_chains.restype = C.c_double
        L.kvo_philox.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _libs[kind] = L
    return _libs[kind]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleModel:
    """Keeps the arrays of one model alive for the C side."""

    def __init__(self, U_up, U_down, bonds, kind="real"):
        self.kind = kind
        dt = np.complex128 if kind == "cplx" else np.float64
        self.U_up = np.ascontiguousarray(U_up, dtype=dt)
        self.U_down = np.ascontiguousarray(U_down, dtype=dt)
        self.bonds = np.ascontiguousarray(np.asarray(bonds, dtype=np.int32).reshape(-1))
        self.N, self.n_up = self.U_up.shape
        self.n_down = self.U_down.shape[1]
        self.c = Model(self.N, self.n_up, self.n_down, len(self.bonds) // 2, _p(self.bonds), _p(self.U_up),
                       _p(self.U_down))
        self.dt = dt

    def refresh(self, U, kappa):
        W = np.zeros((self.N, U.shape[1]), dtype=self.dt)
        ld = C.c_double()
        k = np.ascontiguousarray(kappa, dtype=np.int32)
        sing = lib(self.kind).kvo_refresh(self.N, U.shape[1], _p(np.ascontiguousarray(U, dtype=self.dt)), _p(k), _p(W),
                                          C.byref(ld))
        return W, ld.value, sing

    def new_chain(self, kappa_up, kappa_down, t=0):
        ch = OracleChain(self, kappa_up, kappa_down, t)
        return ch


class OracleChain:
    def __init__(self, model: OracleModel, kappa_up, kappa_down, t=0):
        self.m = model
        self.ku = np.ascontiguousarray(kappa_up, dtype=np.int32).copy()
        self.kd = np.ascontiguousarray(kappa_down, dtype=np.int32).copy()
        self.Wu, ldu, s1 = model.refresh(model.U_up, self.ku)
        self.Wd, ldd, s2 = model.refresh(model.U_down, self.kd)
        self.logdet = (ldu, ldd)
        self.c = Chain(_p(self.ku), _p(self.kd), _p(self.Wu), _p(self.Wd), t, 0, 0.0, 0.0, 0, int(s1 or s2))

    def run(self, seed, walker, n_proposals, refresh_every, measure_every, accept_rule=0, record=True):
        n_e = n_proposals // max(measure_every, 1) + 2 if record else 0
        e = np.zeros(n_e)
        rc = lib(self.m.kind).kvo_run_chain(C.byref(self.m.c), C.byref(self.c), seed, walker, n_proposals,
                                            refresh_every, measure_every, accept_rule, _p(e) if record else None)
        return rc, e

    def local_energy(self):
        return lib(self.m.kind).kvo_local_energy(len(self.m.bonds) // 2, _p(self.m.bonds), _p(self.ku), _p(self.kd),
                                                 _p(self.Wu), self.m.n_up, _p(self.Wd), self.m.n_down)


def run_chains(model: OracleModel, starts, seed, n_proposals, refresh_every, measure_every, accept_rule, n_threads):
    """Runs one chain per start on n_threads host threads; returns (seconds, chains)."""
    chains = [OracleChain(model, ku, kd) for ku, kd in starts]
    arr = (Chain * len(chains))(*[ch.c for ch in chains])
    sec = lib(model.kind).kvo_run_chains(C.byref(model.c), arr, len(chains), seed, n_proposals, refresh_every,
                                         measure_every, accept_rule, n_threads)
    for k, ch in enumerate(chains):
        ch.c = arr[k]
    return sec, chains
