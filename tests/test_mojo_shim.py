"""The Mojo shim (mojo/mojovec_gpu.mojo) against the C header, on the CPU.

No Mojo toolchain is available, so the shim is checked as text: every
`external_call["mv_...", ...](...)` it makes names a function that
include/mojovec_gpu.h declares, with the same number of arguments, and the
shim covers every call CollectionIVFPQ makes into its index (create, train,
add, add_with_ids, nprobe, codebooks, search with and without a filter,
save, load, destroy).
"""

import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _split_args(text):
    """Top-level comma-separated arguments of a call's argument text."""
    out, depth, cur = [], 0, ""
    for ch in text:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _call_args(text, start):
    """The argument text of the call whose '(' is at text[start]."""
    depth = 0
    for i in range(start, len(text)):
        if text[i] == "(":
            depth += 1
        elif text[i] == ")":
            depth -= 1
            if depth == 0:
                return text[start + 1:i]
    raise AssertionError("unbalanced call")


def _header_arity():
    text = open(os.path.join(ROOT, "include", "mojovec_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(mv_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len(_split_args(args))
    return out


def _shim_calls():
    text = open(os.path.join(ROOT, "mojo", "mojovec_gpu.mojo")).read()
    calls = []
    for m in re.finditer(r'external_call\["(mv_[a-z0-9_]+)",\s*[A-Za-z0-9]+\]\(', text):
        args = _call_args(text, m.end() - 1)
        calls.append((m.group(1), len(_split_args(args))))
    return calls


def test_shim_calls_match_header():
    hdr = _header_arity()
    calls = _shim_calls()
    assert calls
    for name, n in calls:
        assert name in hdr, f"{name} is not declared in include/mojovec_gpu.h"
        assert hdr[name] == n, f"{name}: shim passes {n} arguments, header declares {hdr[name]}"


def test_shim_covers_the_collection_call_sites():
    used = {name for name, _ in _shim_calls()}
    for name in ("mv_ctx_create", "mv_ctx_destroy", "mv_ivfpq_create", "mv_ivfpq_destroy",
                 "mv_ivfpq_set_nprobe", "mv_ivfpq_train", "mv_ivfpq_add", "mv_ivfpq_add_with_ids",
                 "mv_ivfpq_set_codebooks", "mv_ivfpq_search", "mv_ivfpq_save_snapshot",
                 "mv_ivfpq_load_snapshot", "mv_ivfpq_snapshot_info", "mv_ivfpq_info",
                 "mv_last_error"):
        assert name in used, name
    text = open(os.path.join(ROOT, "mojo", "mojovec_gpu.mojo")).read()
    assert "filter: Span[UInt8" in text  # the filtered search overload


def test_search_params_field_count():
    """The shim passes mv_search_params as an array of int32 fields."""
    text = open(os.path.join(ROOT, "include", "mojovec_gpu.h")).read()
    body = re.search(r"typedef struct mv_search_params \{(.*?)\} mv_search_params;", text, re.S)
    fields = re.findall(r"int32_t\s+\w+;", re.sub(r"/\*.*?\*/", "", body.group(1), flags=re.S))
    shim = open(os.path.join(ROOT, "mojo", "mojovec_gpu.mojo")).read()
    m = re.search(r"comptime _PARAM_FIELDS = (\d+)", shim)
    assert m and int(m.group(1)) == len(fields)
