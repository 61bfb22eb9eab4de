"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every symbol that
include/pibronic_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re

from conftest import REPO


def declared_symbols():
    text = open(os.path.join(REPO, "include", "pibronic_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|int32_t|int64_t|const char\*)\s+(pbr_\w+)\(", text, re.M)))


def test_header_declares_the_binding_list():
    from pibronic_gb300 import _native
    assert declared_symbols() == sorted(_native.EXPORTED)


def test_library_builds_and_exports_all_symbols():
    from pibronic_gb300 import build, _native
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    lib = _native.load(path)
    assert b"sm_103a" in lib.pbr_version()


def test_product_path_fails_loudly_without_cuda():
    import torch
    from pibronic_gb300 import _native
    if torch.cuda.is_available():
        return
    try:
        _native.require_cuda()
    except RuntimeError as err:
        assert "no CPU fallback" in str(err)
    else:
        raise AssertionError("require_cuda must raise without a device")


def test_calls_with_a_wrong_argument_count_are_rejected():
    """ctypes would pass a surplus argument on silently; the loaded library refuses it before
    anything reaches the native code."""
    import pytest
    from pibronic_gb300 import build, _native
    lib = _native.load(build.build())
    assert lib.pbr_version() is not None
    with pytest.raises(TypeError):
        lib.pbr_version(0)
    with pytest.raises(TypeError):
        lib.pbr_reduce_blocks()


def _fake_models(shapes, variant=0):
    """pbr_model / pbr_outputs arrays for the host-only packer: sizes set, table and output
    pointers non-null but never dereferenced (no device memory on this machine)."""
    from pibronic_gb300 import _native
    M = len(shapes)
    models, outs = (_native.PbrModel * M)(), (_native.PbrOutputs * M)()
    fake = 0x1000
    for i, (A, N, P) in enumerate(shapes):
        m = models[i]
        m.A = m.A_rho = m.n_fill_rho = A
        m.N, m.P, m.K, m.precision, m.variant = N, P, 4, 32, variant
        m.tau, m.delta_beta = 0.01, 1e-3
        for f in ("vib_cs", "vib_th", "vib_c", "vib_d", "vib_e", "vib_l", "vib_qq", "rho_cs", "rho_th",
                  "rho_c", "rho_d", "ring_chol", "src_cdf"):
            setattr(m, f, fake)
        for f in ("s_rho", "s_g", "s_gp", "s_gm"):
            setattr(outs[i], f, fake)
    return models, outs


def _pack(lib, shapes, variant=0, budget=None):
    M = len(shapes)
    models, outs = _fake_models(shapes, variant)
    seeds = (ctypes.c_uint64 * M)(*range(1, M + 1))
    offs = (ctypes.c_uint64 * M)()
    X = (ctypes.c_int64 * M)(*([1000] * M))
    blob = ctypes.create_string_buffer(int(lib.pbr_batch_blob_bytes(M)))
    budgets = None if budget is None else (ctypes.c_int32 * 9)(*budget)
    rc = lib.pbr_batch_pack(models, seeds, offs, X, outs, M, budgets, 0, blob)
    return rc, blob


def test_batch_packing_groups_models_by_kernel_form():
    """The batch packer is host code: models group by surface count, and at 5-6 surfaces by
    whether two tiles fit an SM (the two-block row-team build) -- here 2, 3, 4 surfaces (one
    register-chunk group each), 5 and 6 surfaces at P = 32 (two-block), 6 surfaces at N = 20,
    P = 128 (a 126 KB tile: one-block), 8 surfaces."""
    from pibronic_gb300 import build, _native
    lib = _native.load(build.build())
    shapes = [(2, 4, 16), (3, 6, 32), (4, 12, 64), (5, 16, 32), (6, 10, 32), (6, 20, 128), (8, 8, 32)]
    rc, blob = _pack(lib, shapes)
    assert rc == 0
    assert lib.pbr_batch_groups(blob) == 7
    # two models that share a group stay in one group
    rc, blob = _pack(lib, shapes + [(2, 5, 24), (6, 12, 32)])
    assert rc == 0 and lib.pbr_batch_groups(blob) == 7


def test_batch_packing_rejects_bad_models():
    from pibronic_gb300 import build, _native
    lib = _native.load(build.build())
    rc, _ = _pack(lib, [(4, 12, 2000)])           # more beads than the limit
    assert rc == _native.PBR_ERR_ARG
    rc, _ = _pack(lib, [(9, 4, 16)])              # more surfaces than the row-team form holds
    assert rc != 0


def test_batch_packing_follows_the_per_surface_count_budgets():
    """A negative budget keeps a group of up to 4 surfaces on the register-chunk launches, 0 or a
    positive budget puts it on the row-team form; a budget smaller than one model's one-sample
    tile makes that model take the whole shared memory instead of failing the pack; at 5-6
    surfaces a small budget moves a model into the two-block class (another group)."""
    from pibronic_gb300 import build, _native
    lib = _native.load(build.build())
    shapes = [(2, 4, 16), (4, 12, 64), (6, 20, 128), (6, 10, 32)]
    chunks = [0, -1, -1, -1, -1, 0, 0, 0, 0]
    rc, blob = _pack(lib, shapes, budget=chunks)
    assert rc == 0 and lib.pbr_batch_groups(blob) == 4
    teams = [0, 0, 0, 0, 0, 0, 0, 0, 0]
    rc, blob = _pack(lib, shapes, budget=teams)
    assert rc == 0 and lib.pbr_batch_groups(blob) == 4
    tiny = [0, 4096, 4096, 4096, 4096, 4096, 4096, 4096, 4096]     # below every one-sample tile
    rc, blob = _pack(lib, shapes, budget=tiny)
    assert rc == 0
    small = [0, -1, -1, -1, -1, 72 * 1024, 72 * 1024, 0, 0]
    rc, blob = _pack(lib, [(6, 20, 128), (6, 20, 64)], budget=small)
    assert rc == 0 and lib.pbr_batch_groups(blob) >= 1
