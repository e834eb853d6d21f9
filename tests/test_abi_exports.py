"""The C-ABI library loads without a GPU and exports every function the public headers declare
(no compute calls: none of these tests needs a device)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("halcuda.h", "ringcuda.h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:hc_status|size_t|int64_t|int|double|uint64_t|const char\s*\*|void)\s*\**\s*(hc_\w+)\s*\(",
                             text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_the_backend_surface():
    names = declared_functions()
    # one entry per hal::Backend method family (src/hal/mod.rs:108-350) and the ring/BFV layer
    for must in ("hc_allocate_i64", "hc_import", "hc_export", "hc_ntt_mul_mont64_dim", "hc_inner_product_i64",
                 "hc_bconv_correct_pow2_wide", "hc_permute", "hc_bfv_hom_mul", "hc_bfv_hom_gal",
                 "hc_crt_batch_run", "hc_dbfv_hom_cyclic_transform", "hc_keyset_create", "hc_bfv_key_switch_noalloc"):
        assert must in names, must
    assert len(names) > 90


def test_library_exports_every_declared_function():
    import halcuda

    path = halcuda.lib_path() if hasattr(halcuda, "lib_path") else None
    if path is None:
        pytest.skip("library path helper missing")
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_rust_binding_declares_only_exported_functions():
    """The Rust `hal::cuda` module (include/hal_cuda.rs) binds only functions the C headers declare,
    with the headers' parameter counts."""
    text = open(os.path.join(ROOT, "include", "hal_cuda.rs")).read()
    rust = {}
    for m in re.finditer(r"fn (hc_\w+)\s*\(([^)]*)\)", text, flags=re.S):
        params = [p for p in m.group(2).split(",") if p.strip()]
        rust[m.group(1)] = len(params)
    assert len(rust) >= 30
    c = {}
    for h in HEADERS:
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"(hc_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
            params = [p for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
            c.setdefault(m.group(1), len(params))
    for name, n in sorted(rust.items()):
        assert name in c, name
        assert c[name] == n, (name, c[name], n)
