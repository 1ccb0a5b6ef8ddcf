"""Band / group-velocity serving over the C ABI server (uepm_server_*), the mixed-material context set of
the uneven-batch workload, and the seeded Poisson load of the serving benchmark.

    python -m ultimateepm_gb300.serve --rates 100,500 --requests 200 [--kmax 50000] [--no-velocity]

The server (csrc/server.cu) keeps the contexts resident, cuts requests into work items, admits them
by device-memory footprint and runs them on several streams at once (continuous batching). This
module adds the host-side conveniences: output arrays per request, and a load generator that submits
requests at Poisson arrival times (seeded), each for a random context of the set, with a log-uniform
number of k-points, and reports the latency percentiles and throughput the server measured.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import time
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .api import Materials, _Context, generate_basis_vectors

HERE = os.path.dirname(os.path.abspath(__file__))
PARAMS = os.path.join(os.path.dirname(HERE), "params")

# The uneven mixed-material set: 8 diamond / zinc-blende materials, cutoffs of 8..13 shells (basis
# 89..229), spin-orbit on for the four whose spin-orbit parameters the reference's functional
# supports (periods 2..4), giving matrix orders 89..458. (symbol, shells, soc)
MIXED_SET = [
    ("Si", 10, True), ("Ge", 12, True), ("GaAs", 8, True), ("GaP", 13, True),
    ("Sn", 11, False), ("InP", 9, False), ("InAs", 13, False), ("AlAs", 8, False),
]


def make_contexts(precision: int = N.UEPM_PREC_MIXED, groups=MIXED_SET, yaml: str | None = None) -> list[_Context]:
    """One resident context per (material, cutoff, SOC) group; nonlocal corrections on where the
    material has them."""
    mats = Materials()
    mats.load_material_parameters(yaml or os.path.join(PARAMS, "materials.yaml"))
    out = []
    for sym, shells, soc in groups:
        m = mats.materials[sym]
        out.append(_Context(m, generate_basis_vectors(shells), bool(m.raw.has_nonlocal), soc, precision))
    return out


def sample_bz(n: int, rng: np.random.Generator) -> np.ndarray:
    """Uniform k in the first Brillouin zone (|k_i| <= 1, |kx| + |ky| + |kz| <= 3/2), reduced units."""
    out = np.empty((0, 3))
    while len(out) < n:
        c = rng.uniform(-1.0, 1.0, size=(2 * (n - len(out)) + 8, 3))
        out = np.concatenate([out, c[np.abs(c).sum(axis=1) <= 1.5]])
    return np.ascontiguousarray(out[:n])


@dataclass
class Ticket:
    id: int
    E: np.ndarray
    V: np.ndarray | None
    status: np.ndarray
    k: np.ndarray


class Server:
    """A query server over resident contexts (see include/uepm_gb300.h for the scheduling rules)."""

    def __init__(self, contexts: list[_Context], hbm_budget: int = 8 << 30, slots: int = 4, max_chunk: int = 2048,
                 max_nb: int = 32):
        self.L = N.load()
        self.contexts = contexts
        arr = (C.c_void_p * len(contexts))(*[c.h for c in contexts])
        h = C.c_void_p()
        N.check(self.L.uepm_server_create(arr, len(contexts), hbm_budget, slots, max_chunk, max_nb, C.byref(h)))
        self.h = h
        self._live: dict[int, Ticket] = {}

    def submit(self, ctx_index: int, k: np.ndarray, nb: int, velocity: bool = False, h: float = 1e-4) -> Ticket:
        k = np.ascontiguousarray(k, dtype=np.float64).reshape(-1, 3)
        nk = len(k)
        E = np.zeros((nk, nb))
        V = np.zeros((nk, nb, 3)) if velocity else None
        st = np.zeros(nk, dtype=np.int32)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None
        rid = self.L.uepm_server_submit(self.h, ctx_index, dp(k), nk, nb, N.UEPM_SERVE_VELOCITY if velocity else 0, h,
                                        dp(E), dp(V), st.ctypes.data_as(C.POINTER(C.c_int32)))
        N.check(int(rid))
        t = Ticket(int(rid), E, V, st, k)  # keeps the buffers alive until the wait
        self._live[t.id] = t
        return t

    def wait(self, t: Ticket, timeout: float = -1.0) -> bool:
        rc = self.L.uepm_server_wait(self.h, t.id, timeout)
        if rc == 1:
            return False
        self._live.pop(t.id, None)
        N.check(rc)
        return True

    def stats(self) -> dict:
        p50, p99, span = C.c_double(), C.c_double(), C.c_double()
        done, kp = C.c_uint64(), C.c_uint64()
        N.check(self.L.uepm_server_stats(self.h, C.byref(p50), C.byref(p99), C.byref(done), C.byref(kp), C.byref(span)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "completed": done.value, "k_points": kp.value,
                "span_s": span.value}

    def reset_stats(self):
        N.check(self.L.uepm_server_reset_stats(self.h))

    def close(self):
        if self.h:
            self.L.uepm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_requests(n: int, rate: float, seed: int, ngroups: int, kmin: int = 1, kmax: int = 50000,
                     nb_range=(8, 16)) -> list[tuple[float, int, int, int]]:
    """(arrival time s, group, k-points, bands) of n requests: exponential inter-arrival times of mean
    1 / rate, groups uniform, k-point counts log-uniform in [kmin, kmax], bands uniform in nb_range."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    g = rng.integers(0, ngroups, size=n)
    nk = np.exp(rng.uniform(math.log(kmin), math.log(kmax + 1), size=n)).astype(np.int64)
    nk = np.clip(nk, kmin, kmax)
    nb = rng.integers(nb_range[0], nb_range[1] + 1, size=n)
    return [(float(a), int(b), int(c), int(d)) for a, b, c, d in zip(t, g, nk, nb)]


def run_load(server: Server, requests, seed: int = 0, velocity: bool = True, h: float = 1e-4) -> dict:
    """Submits the requests at their arrival times (k-points drawn beforehand), waits for all of them,
    and returns the server's statistics with the offered load."""
    rng = np.random.default_rng(seed + 1)
    ks = [sample_bz(nk, rng) for _, _, nk, _ in requests]
    server.reset_stats()
    t0 = time.perf_counter()
    tickets = []
    for (ta, g, nk, nb), k in zip(requests, ks):
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        tickets.append(server.submit(g, k, nb, velocity=velocity, h=h))
    for t in tickets:
        server.wait(t)
    wall = time.perf_counter() - t0
    bad = int(sum(int(t.status.any()) for t in tickets))
    s = server.stats()
    span = requests[-1][0] if requests else 0.0
    s.update({"requests": len(requests), "offered_req_per_s": len(requests) / span if span > 0 else None,
              "k_points_per_s": s["k_points"] / s["span_s"] if s["span_s"] > 0 else None,
              "solves_per_k_point": 7 if velocity else 1, "wall_s": wall, "requests_with_nonzero_status": bad})
    return s


def main(argv=None) -> int:
    p = argparse.ArgumentParser(description="Poisson load against the band / velocity server (one GPU)")
    p.add_argument("--rates", default="100", help="comma-separated request rates (req/s)")
    p.add_argument("--requests", type=int, default=200)
    p.add_argument("--kmin", type=int, default=1)
    p.add_argument("--kmax", type=int, default=50000)
    p.add_argument("--no-velocity", action="store_true")
    p.add_argument("--fd-step", type=float, default=1e-4)
    p.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    p.add_argument("--slots", type=int, default=4)
    p.add_argument("--hbm-gb", type=float, default=32.0)
    p.add_argument("--max-chunk", type=int, default=2048)
    p.add_argument("--seed", type=int, default=20261203)
    a = p.parse_args(argv)
    prec = N.UEPM_PREC_MIXED if a.precision == "mixed" else N.UEPM_PREC_FP64
    ctxs = make_contexts(prec)
    srv = Server(ctxs, hbm_budget=int(a.hbm_gb * (1 << 30)), slots=a.slots, max_chunk=a.max_chunk)
    try:
        for rate in [float(r) for r in a.rates.split(",")]:
            reqs = poisson_requests(a.requests, rate, a.seed, len(ctxs), a.kmin, a.kmax)
            res = run_load(srv, reqs, seed=a.seed, velocity=not a.no_velocity, h=a.fd_step)
            res.update({"rate": rate, "kmin": a.kmin, "kmax": a.kmax, "precision": a.precision})
            print(json.dumps(res), flush=True)
    finally:
        srv.close()
        for c in ctxs:
            c.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
