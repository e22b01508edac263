"""The precision form with its fallback: a wave run in FP16 delta storage
that moves to the compensated FP16 + int8 form when its drift against a
reference run exceeds a stated tolerance.

    run = GuardedWave(grid, 25, tol=1e-3, dt=5e-4, src=...)
    run.upload(v, s, u)
    for _ in range(100):
        run.iterate(10)
        ref.iterate(10)                  # e.g. the FP64 run of the same workload
        run.check(ref)                   # relative L2 of u; moves past margin * tol

The move happens at the first check whose error exceeds ``margin * tol``
(half the tolerance by default): the error reached before the move stays in
the state the fallback continues from, so the margin is what is left for the
fallback's own drift.  FP16 storage of u rounds it every step, which makes
its error grow about as sqrt(steps) from the start; checks early in a run
have to be frequent enough to catch the crossing of the margin.

The move creates a context of the fallback storage, sets s there the way it
was set (the uploaded array or the same fill) and takes u, v and the source
clock over from the running context on the device (``st3d_transfer``: the
values a download returns, re-encoded).  Everything runs through the C ABI;
the reference run is whatever context the caller compares with.
"""
from . import api


class GuardedWave:
    def __init__(self, grid, points, tol=1e-3, storage="f16", fallback="f16_hilo", margin=0.5, **kw):
        if not 0.0 < margin <= 1.0:
            raise ValueError("margin must be in (0, 1]")
        self.grid, self.points, self.tol, self.margin = grid, points, float(tol), float(margin)
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
        """Relative L2 of u against `ref`'s u; past margin * tol the run moves
        to the fallback storage (once).  Returns the error."""
        err = self.st.rel_l2(ref)
        self.history.append((self.steps, self.current_storage, err))
        if err > self.margin * self.tol and self.switched_at is None:
            self._move()
        return err

    def _move(self):
        nxt = api.Stencil(self.grid, self.points, "wave", self.fallback, **self.kw)
        try:
            # s first: upload and fill reset the clock the transfer carries over
            if self._s is None:
                nxt.fill(api.FIELD_S, api.FILL_CONST, 0, 0.0)
            elif self._s[0] == "array":
                nxt.upload(None, self._s[1], None)
            else:
                nxt.fill(api.FIELD_S, *self._s[1:])
            nxt.transfer_from(self.st)
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
