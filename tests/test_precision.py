"""The guarded precision run's host logic without a GPU: a fake context
replaces the library's, scripted errors drive the checks."""
import numpy as np
import pytest

from stencil3d_gb300 import api, precision


class FakeStencil:
    log = []
    errors = []

    def __init__(self, grid, points, mode, storage, **kw):
        self.storage, self.kw, self.closed = storage, kw, False
        FakeStencil.log.append(("create", storage))

    def upload(self, v=None, s=None, u=None):
        FakeStencil.log.append(("upload", self.storage, v is not None, s is not None, u is not None))

    def fill(self, field, kind, seed=0, a=0.0, b=0.0):
        FakeStencil.log.append(("fill", self.storage, field, kind, seed, a, b))

    def iterate(self, n):
        FakeStencil.log.append(("iterate", self.storage, n))

    def rel_l2(self, ref):
        return FakeStencil.errors.pop(0)

    def transfer_from(self, src):
        FakeStencil.log.append(("transfer", self.storage, src.storage))

    def close(self):
        self.closed = True
        FakeStencil.log.append(("close", self.storage))


@pytest.fixture
def fake(monkeypatch):
    monkeypatch.setattr(api, "Stencil", FakeStencil)
    FakeStencil.log, FakeStencil.errors = [], []
    return FakeStencil


def test_moves_once_past_the_margin(fake):
    run = precision.GuardedWave(None, 25, tol=1e-3, dt=5e-4)
    run.fill(api.FIELD_S, api.FILL_CONST, 0, 0.0)
    fake.errors[:] = [2e-4, 4.9e-4, 5.1e-4, 9e-4, 2e-3]
    for _ in range(5):
        run.iterate(10)
        run.check("ref")
    assert run.switched_at == 30 and run.current_storage == "f16_hilo"
    assert [h[1] for h in run.history] == ["f16", "f16", "f16", "f16_hilo", "f16_hilo"]
    # the move: new context, s set the way it was set (a fill), then the transfer
    i = fake.log.index(("create", "f16_hilo"))
    assert fake.log[i + 1] == ("fill", "f16_hilo", api.FIELD_S, api.FILL_CONST, 0, 0.0, 0.0)
    assert fake.log[i + 2] == ("transfer", "f16_hilo", "f16")
    assert ("close", "f16") in fake.log
    # past the tolerance after the move: no second move
    assert fake.log.count(("create", "f16_hilo")) == 1


def test_uploaded_s_is_uploaded_again(fake):
    run = precision.GuardedWave(None, 13, tol=1e-2, fallback="f16_hl", margin=1.0)
    s = np.zeros(8, np.float32)
    run.upload(None, s, None)
    fake.errors[:] = [1.1e-2]
    run.iterate(4)
    run.check("ref")
    i = fake.log.index(("create", "f16_hl"))
    assert fake.log[i + 1] == ("upload", "f16_hl", False, True, False)
    assert fake.log[i + 2] == ("transfer", "f16_hl", "f16")
    assert run.switched_at == 4


def test_margin_is_checked():
    with pytest.raises(ValueError):
        precision.GuardedWave(None, 7, margin=0.0)
    with pytest.raises(ValueError):
        precision.GuardedWave(None, 7, margin=1.5)
