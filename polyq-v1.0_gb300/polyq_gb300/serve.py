"""Python front-end of the serving loop (pq_server_*): continuous batching over resident
simulators with memory-based admission; every result carries submit/completion times."""
from __future__ import annotations

import ctypes as ct

from . import _native as N

AMPLITUDE, PROBABILITY, MARGINAL = 0, 1, 2
M64 = 0xFFFFFFFFFFFFFFFF


class Server:
    def __init__(self, sims, max_slots=256, mem_budget_bytes=1 << 30, max_branch_dim=40):
        self._L = N.lib()
        self.sims = list(sims)
        arr = (ct.c_void_p * len(self.sims))(*[s.handle for s in self.sims])
        h = ct.c_void_p()
        N.check(self._L.pq_server_create(len(self.sims), arr, int(max_slots), int(mem_budget_bytes),
                                         int(max_branch_dim), ct.byref(h)))
        self._h = h
        self.max_slots = max_slots

    def set_pieces(self, split_log2=28, piece_log2=32):
        """Requests above 2^split_log2 branches run in the background in pieces of at most
        2^piece_log2 branches (pq_server_set_pieces)."""
        N.check(self._L.pq_server_set_pieces(self._h, int(split_log2), int(piece_log2)))

    def now(self) -> float:
        return float(self._L.pq_server_now(self._h))

    def submit(self, requests):
        """requests: iterables of dicts {sim, kind, x, y | qubit, outcome, tag}."""
        reqs = list(requests)
        arr = (N.Request * max(1, len(reqs)))()
        for i, r in enumerate(reqs):
            q = arr[i]
            q.sim = int(r["sim"])
            q.kind = int(r.get("kind", AMPLITUDE))
            x = int(r.get("x", 0))
            y = int(r.get("y", 0))
            q.x[0], q.x[1] = x & M64, (x >> 64) & M64
            q.y[0], q.y[1] = y & M64, (y >> 64) & M64
            q.qubit = int(r.get("qubit", 0))
            q.outcome = int(r.get("outcome", 0))
            q.tag = int(r.get("tag", i))
        N.check(self._L.pq_server_submit(self._h, len(reqs), arr))

    def poll(self, cap=4096, timeout_s=0.0):
        buf = (N.Result * cap)()
        k = int(self._L.pq_server_poll(self._h, buf, cap, float(timeout_s)))
        out = []
        for i in range(k):
            r = buf[i]
            out.append({"tag": r.tag, "status": r.status, "kind": r.kind, "re": r.re, "im": r.im,
                        "errbound": r.errbound, "submit_s": r.submit_s, "done_s": r.done_s, "level": r.level,
                        "pieces": r.pieces})
        return out

    def drain(self, timeout_s=60.0):
        N.check(self._L.pq_server_drain(self._h, float(timeout_s)))

    def collect(self, n, timeout_s=60.0):
        """Poll until n results arrived (or the timeout)."""
        import time
        res = []
        t_end = time.monotonic() + timeout_s
        while len(res) < n and time.monotonic() < t_end:
            res.extend(self.poll(4096, 0.05))
        return res

    def close(self):
        if getattr(self, "_h", None):
            self._L.pq_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
