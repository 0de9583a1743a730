"""CPU checks of the C-ABI library: it builds, loads without a GPU, exports
every function include/mojovec_gpu.h declares, and the Python binding
declares exactly those signatures. No compute calls are made here."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "mojovec_gpu.h")).read()
    return sorted(set(re.findall(r"\b(mv_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_hot_path():
    names = _declared()
    for required in ("mv_ivfpq_search", "mv_ivfpq_train", "mv_ivfpq_add_with_ids", "mv_flat_search",
                     "mv_sq8_search", "mv_kmeans_train", "mv_pq_encode", "mv_pq_train",
                     "mv_sq8_encode", "mv_normalize"):
        assert required in names


def test_library_exports_every_declared_symbol(mv):
    lib = ctypes.CDLL(os.path.join(ROOT, "mojovec_gb300", "libmojovec_gpu.so"))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from mojovec_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == _declared()


def test_stage_names_follow_header_stage_ids():
    """The binding's stage names index mv_ctx_stage_times' arrays, so their
    order must be the header's MV_STAGE_* ids."""
    from mojovec_gb300 import _lib

    text = open(os.path.join(ROOT, "include", "mojovec_gpu.h")).read()
    ids = {name.lower(): int(v) for name, v in re.findall(r"#define MV_STAGE_([A-Z]+) (\d+)", text)}
    count = ids.pop("count")
    assert count == len(_lib.STAGES) == len(ids)
    assert all(ids[name] == i for i, name in enumerate(_lib.STAGES))


def test_version_and_error_without_gpu(mv):
    from mojovec_gb300 import _lib

    lib = _lib.load()
    assert lib.mv_version().startswith(b"mojovec-gb300")
    h = ctypes.c_void_p()
    st = lib.mv_ctx_create(0, ctypes.byref(h))
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert st != 0
        assert _lib.last_error()
    else:
        assert st == 0
        lib.mv_ctx_destroy(h)


def test_null_arguments_are_rejected(mv):
    from mojovec_gb300 import _lib

    lib = _lib.load()
    assert lib.mv_ivfpq_search(None, None, 1, 10, None, 0, None, None, None) == _lib.MV_ERR_ARG
    assert lib.mv_flat_add(None, None, 1) == _lib.MV_ERR_ARG
    assert lib.mv_ctx_create(0, None) == _lib.MV_ERR_ARG
