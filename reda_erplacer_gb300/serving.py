"""Continuous-batching placement server (erp_server_* in include/erplacer.h)
and an open-loop driver for a stream of timed job arrivals."""
import ctypes as C
import time

import numpy as np

from . import lib as L
from .lib import JobResult, ServerParams


class Server:
    def __init__(self, max_active=64, hbm_budget_gb=150.0, max_iterations=600, stop_overflow=0.10,
                 chunk=8, keep_positions=False, device=0):
        self.lib = L.load()
        p = ServerParams(int(device), int(max_active), int(hbm_budget_gb * 2 ** 30), int(max_iterations),
                         float(stop_overflow), int(chunk), 1 if keep_positions else 0)
        h = C.c_void_p()
        L.check(self.lib.erp_server_create(C.byref(p), C.byref(h)))
        self.h = h
        self._sizes = {}

    def _ck(self, st):
        if st != L.OK:
            raise L.ErpError(st, self.lib.erp_server_last_error(self.h).decode(errors="replace"))

    def submit(self, job_id, design, num_bins, target_density=1.0, start_mode=L.START_DB):
        s = design.to_struct()
        prm = L.Params(int(num_bins[0]), int(num_bins[1]), float(target_density), int(start_mode),
                       L.PREC_FP32, 0, None, 0)
        self._ck(self.lib.erp_server_submit(self.h, int(job_id), C.byref(s), C.byref(prm)))
        self._sizes[int(job_id)] = int(design.num_nodes)

    def pump(self):
        a, q = C.c_int32(), C.c_int32()
        self._ck(self.lib.erp_server_pump(self.h, C.byref(a), C.byref(q)))
        return a.value, q.value

    def cancel(self, job_id):
        """Withdraw a queued or running job (erp_server_cancel); its result
        carries ECANCELED."""
        self._ck(self.lib.erp_server_cancel(self.h, int(job_id)))

    def poll(self):
        buf = (JobResult * 256)()
        out = []
        while True:
            n = C.c_int32()
            self._ck(self.lib.erp_server_poll(self.h, buf, 256, C.byref(n)))
            out.extend(buf[i].as_dict() for i in range(n.value))
            if n.value < 256:
                return out

    def positions(self, job_id):
        N = self._sizes[int(job_id)]
        x = np.empty(N, np.float32)
        y = np.empty(N, np.float32)
        self._ck(self.lib.erp_server_positions(self.h, int(job_id), x.ctypes.data_as(L.f32p),
                                               y.ctypes.data_as(L.f32p)))
        return x, y

    def now(self):
        return float(self.lib.erp_server_now(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.erp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_footprint(design, num_bins):
    lib = L.load()
    s = design.to_struct()
    prm = L.Params(int(num_bins[0]), int(num_bins[1]), 1.0, 0, L.PREC_FP32, 0, None, 0)
    b = C.c_int64()
    L.check(lib.erp_estimate_footprint(C.byref(s), C.byref(prm), C.byref(b)))
    return int(b.value)


def run_stream(server, jobs, arrivals):
    """Open-loop driver: jobs[i] = (design, bins) is submitted when the server
    clock passes arrivals[i] (seconds from the start); the server is pumped
    until every job has finished.  Returns the results with latency added."""
    order = np.argsort(arrivals, kind="stable")
    t_start = server.now()
    nxt = 0
    results = []
    while len(results) < len(jobs):
        now = server.now() - t_start
        while nxt < len(order) and arrivals[order[nxt]] <= now:
            i = int(order[nxt])
            design, bins = jobs[i]   # fetched once (jobs may be generated lazily)
            server.submit(i, design, bins)
            del design
            nxt += 1
        active, queued = server.pump()
        results.extend(server.poll())
        if active == 0 and queued == 0 and nxt < len(order):   # idle until the next arrival
            wait = arrivals[order[nxt]] - (server.now() - t_start)
            if wait > 0:
                time.sleep(min(wait, 0.05))
    for r in results:
        r["latency_s"] = r["finish_s"] - r["submit_s"]
    return results
