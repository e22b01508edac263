"""The precision form with its fallback: a wave run in FP16 delta storage
that moves to the compensated FP16 + int8 form when its drift against a
reference run exceeds a stated tolerance.

    run = GuardedWave(grid, 25, tol=1e-3, dt=5e-4, src=...)
    run.upload(v, s, u)
    for _ in range(10):
        run.iterate(100)
        ref.iterate(100)                 # e.g. the FP64 run of the same workload
        run.check(ref)                   # relative L2 of u; falls back past tol

The move downloads u and v (the values a download returns), uploads them
into a context of the fallback storage, sets s again the way it was set
(the uploaded array or the same fill) and carries the source clock over
(``set_step``).  Everything runs through the C ABI; the reference run is
whatever context the caller compares with.
"""
from . import api


class GuardedWave:
    def __init__(self, grid, points, tol=1e-3, storage="f16", fallback="f16_hilo", **kw):
        self.grid, self.points, self.tol = grid, points, float(tol)
        self.storage, self.fallback, self.kw = storage, fallback, dict(kw)
        self.st = api.Stencil(grid, points, "wave", storage, **kw)
        self.steps = 0
        self.switched_at = None
        self.history = []   # (step, storage, relative L2 of u)
        self._s = None      # how s was set: ("array", copy) or ("fill", kind, seed, a, b)

    @property
    def current_storage(self):
        return self.storage if self.switched_at is None else self.fallback

    def upload(self, v=None, s=None, u=None):
        self.st.upload(v, s, u)
        if s is not None:
            self._s = ("array", s.copy())
        self.steps = 0

    def fill(self, field, kind, seed=0, a=0.0, b=0.0):
        self.st.fill(field, kind, seed, a, b)
        if field == api.FIELD_S:
            self._s = ("fill", kind, seed, a, b)
        self.steps = 0

    def iterate(self, n):
        self.st.iterate(n)
        self.steps += int(n)

    def synchronize(self):
        self.st.synchronize()

    def download(self, v=None, u=None):
        self.st.download(v, u)

    def check(self, ref):
        """Relative L2 of u against `ref`'s u; past the tolerance the run moves
        to the fallback storage (once).  Returns the error."""
        err = self.st.rel_l2(ref)
        self.history.append((self.steps, self.current_storage, err))
        if err > self.tol and self.switched_at is None:
            self._move()
        return err

    def _move(self):
        g = self.grid
        u, v = g.empty(), g.empty()
        self.st.download(v, u)
        self.st.synchronize()
        nxt = api.Stencil(g, self.points, "wave", self.fallback, **self.kw)
        try:
            nxt.upload(v, None, u)
            if self._s is None:
                nxt.fill(api.FIELD_S, api.FILL_CONST, 0, 0.0)
            elif self._s[0] == "array":
                nxt.upload(None, self._s[1], None)
            else:
                nxt.fill(api.FIELD_S, *self._s[1:])
            nxt.set_step(self.steps)
        except api.St3dError:
            nxt.close()
            raise
        self.st.close()
        self.st = nxt
        self.switched_at = self.steps

    def close(self):
        self.st.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
