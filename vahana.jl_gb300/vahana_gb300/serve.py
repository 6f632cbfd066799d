"""Serving loop over libvahana_gb300: jobs of the SIR and the opinion test
model arrive over time and are stepped together, one launch per model per
tick, each job's result equal to running it alone (no reference
counterpart; the reference runs one simulation per process)."""
import ctypes as C

import numpy as np

from ._lib import check, lib

SIR, OPINION = 0, 1


class JobSpec(C.Structure):
    _fields_ = [("model", C.c_int), ("n", C.c_uint64), ("mean_degree", C.c_double),
                ("steps", C.c_int32), ("seed", C.c_uint64), ("beta", C.c_double),
                ("recovery", C.c_int32), ("eps", C.c_double), ("wmax", C.c_double),
                ("keep_state", C.c_int), ("fail_build", C.c_int)]


class JobResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("model", C.c_int), ("n", C.c_uint64), ("steps", C.c_int32),
                ("arrival_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double),
                ("checksum", C.c_uint64), ("summary", C.c_double),
                ("device_bytes", C.c_uint64), ("status", C.c_int), ("error", C.c_char * 124)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["error"] = self.error.decode(errors="replace")
        return d


def sir_job(n, degree=10, steps=50, seed=1, beta=0.05, recovery=7, keep_state=False):
    """The job of models.build_sir(n, degree, beta, recovery, seed) run for `steps`."""
    return JobSpec(model=SIR, n=n, mean_degree=float(degree), steps=steps, seed=seed, beta=beta,
                   recovery=recovery, eps=0.0, wmax=0.0, keep_state=int(keep_state))


def opinion_job(n, mean_degree=20, steps=50, seed=1, eps=0.3, wmax=1e4, keep_state=False):
    """The job of models.build_opinion(n, mean_degree, 2.5, wmax, eps, seed) run for `steps`."""
    return JobSpec(model=OPINION, n=n, mean_degree=float(mean_degree), steps=steps, seed=seed,
                   beta=0.0, recovery=0, eps=eps, wmax=wmax, keep_state=int(keep_state))


class Server:
    def __init__(self, budget_bytes=64 << 30, max_active=1024):
        h = C.c_void_p()
        check(lib().vg_serve_create(int(budget_bytes), int(max_active), C.byref(h)))
        self._h = h

    def submit(self, spec):
        i = C.c_int64()
        check(lib().vg_serve_submit(self._h, C.byref(spec), C.byref(i)))
        return i.value

    def poll(self, cap=1024):
        out = (JobResult * cap)()
        n = C.c_uint64()
        check(lib().vg_serve_poll(self._h, out, cap, C.byref(n)))
        return [out[k].as_dict() for k in range(n.value)]

    def job_state(self, job_id, spec):
        n = C.c_uint64()
        check(lib().vg_serve_job_state(self._h, job_id, None, 0, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        check(lib().vg_serve_job_state(self._h, job_id, buf.ctypes.data, buf.nbytes, C.byref(n)))
        if spec.model == SIR:
            return buf[:spec.n].copy(), buf[spec.n:].view(np.int32).copy()
        return buf.view(np.float64).copy()

    def stats(self):
        v = [C.c_uint64() for _ in range(6)]
        check(lib().vg_serve_stats(self._h, *[C.byref(x) for x in v]))
        return dict(zip(["queued", "active", "done", "ticks", "sim_steps", "bytes_in_use"],
                        [x.value for x in v]))

    def drain(self):
        check(lib().vg_serve_drain(self._h))

    def close(self):
        if self._h:
            check(lib().vg_serve_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
