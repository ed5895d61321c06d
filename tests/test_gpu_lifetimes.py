"""Field storage from the context's stream-ordered pool: creating and
destroying fields reuses the pool's blocks (device memory stays bounded),
data written before a destroy is not corrupted by a later allocation, and a
field destroyed after its context is released without touching the
context (~Field and the context's lifetime, src/focss/field.cpp:130,
543-547)."""
import numpy as np
import pytest

import focss_gb300 as fg

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def test_create_destroy_cycles_reuse_the_pool():
    ctx = fg.Context(0)
    try:
        n, b = 1 << 20, 8  # 64 MB per field
        keep = fg.Field(fg.Domain(1, n, 1e-12), batch=b, ctx=ctx)
        ctx.sync()
        free0 = torch.cuda.mem_get_info(0)[0]
        for i in range(50):
            f = fg.Field(fg.Domain(1, n, 1e-12), batch=b, ctx=ctx)
            f *= 1.0
            f.close()
        ctx.sync()
        # one or two blocks' worth of pool growth at most, not 50
        assert free0 - torch.cuda.mem_get_info(0)[0] <= 3 * 64 * 2 ** 20
        keep.close()
    finally:
        ctx.close()


def test_data_survives_neighbouring_allocations():
    ctx = fg.Context(0)
    try:
        rng = np.random.default_rng(3)
        x = (rng.standard_normal((2, 1, 4096)) + 1j * rng.standard_normal((2, 1, 4096))).astype(np.complex64)
        a = fg.Field(fg.Domain(1, 4096, 1e-12), data=x, batch=2, ctx=ctx)
        for _ in range(20):
            t = fg.Field(fg.Domain(1, 4096, 1e-12), batch=2, ctx=ctx)  # zero-filled on creation
            assert not np.any(t.numpy())
            t.close()
        assert np.array_equal(a.numpy(), x.astype(complex))
    finally:
        ctx.close()


def test_field_destroyed_after_its_context():
    ctx = fg.Context(0)
    f = fg.Field(fg.Domain(1, 1 << 12, 1e-12), batch=2, ctx=ctx)
    ctx.close()
    f.close()  # released without the context
