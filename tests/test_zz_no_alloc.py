"""The allocation-free reduction entry point, pbr_reduce_terms_static.

Some callers cannot allocate device memory: a plain FFI caller with no GPU array library, or one
whose device memory is held by its own pool and that must not call cudaMalloc/cudaFree.  This
entry point takes no scratch buffer; its partial sums live in a fixed device array inside the
library.  The test calls it through the C ABI and checks it against pbr_reduce_terms (which takes
caller scratch) on two calls in a row with different inputs, so a stale array from the first call
would show, and checks that a request above the fixed capacity is refused without a launch.
It lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

RTOL = 1e-12     # same partition, same merge order as pbr_reduce_terms: equal up to rounding


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pibronic_gb300 import build, _native
    return _native.load(build.build())


def _inputs(seed, X):
    g = torch.Generator(device="cpu").manual_seed(seed)
    rho = torch.rand(X, generator=g, dtype=torch.float64) + 0.5
    gg = rho * (1.0 + 0.3 * torch.randn(X, generator=g, dtype=torch.float64))
    gp = gg * (1.0 + 1e-3 * torch.randn(X, generator=g, dtype=torch.float64))
    gm = gg * (1.0 - 1e-3 * torch.randn(X, generator=g, dtype=torch.float64))
    return [t.cuda() for t in (rho, gg, gp, gm)]


def _with_scratch(lib, arrs, X, db):
    from pibronic_gb300 import _native
    nb = int(lib.pbr_reduce_blocks(X))
    scratch = torch.empty(9 * nb, dtype=torch.float64, device="cuda")
    out = torch.empty(7, dtype=torch.float64, device="cuda")
    p = _native.ptr
    _native.check(lib.pbr_reduce_terms(*[p(a) for a in arrs], X, db, p(scratch), p(out),
                                       _native.stream_handle()), "pbr_reduce_terms")
    return out.cpu().numpy()


def _static(lib, arrs, X, db):
    from pibronic_gb300 import _native
    out = torch.empty(7, dtype=torch.float64, device="cuda")
    p = _native.ptr
    rc = lib.pbr_reduce_terms_static(*[p(a) for a in arrs], X, db, p(out), _native.stream_handle())
    _native.check(rc, "pbr_reduce_terms_static")
    return out.cpu().numpy()


def test_static_matches_scratch_version_two_calls_in_a_row(lib):
    X, db = 3_000_000, 3.9e-3
    first = _inputs(1, X)
    second = _inputs(2, X)
    a1, b1 = _static(lib, first, X, db), _with_scratch(lib, first, X, db)
    a2, b2 = _static(lib, second, X, db), _with_scratch(lib, second, X, db)
    torch.cuda.synchronize()
    assert np.allclose(a1, b1, rtol=RTOL, atol=0)
    assert np.allclose(a2, b2, rtol=RTOL, atol=0)
    assert not np.allclose(a1, a2)           # the second call did not reuse the first's sums
    assert a1[0] == X and a2[0] == X


def test_static_refuses_more_than_its_capacity(lib):
    from pibronic_gb300 import _native
    cap = int(lib.pbr_reduce_terms_static_max_samples())
    assert cap == 1024 * 4096
    arrs = _inputs(3, 8)
    out = torch.full((7,), -1.0, dtype=torch.float64, device="cuda")
    rc = lib.pbr_reduce_terms_static(*[_native.ptr(a) for a in arrs], cap + 1, 1e-3,
                                     _native.ptr(out), _native.stream_handle())
    assert rc == _native.PBR_ERR_CAPACITY
    assert torch.all(out == -1.0)            # nothing was launched
