"""C-ABI library checks that need no GPU: it loads, exports every function
declared in include/*.h, and fails cleanly (EINVAL + message) without a GPU."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in ("gpuspatial_c.h", "spj_gb300.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"struct\s+\w+\s*\{.*?\};", "", src, flags=re.S)
        # top-level declarations start in column 0: "<type> <name>("
        for m in re.finditer(r"^(?:const\s+)?(?:struct\s+)?[A-Za-z_]\w*[\s\*]+([A-Za-z_]\w*)\s*\(",
                             src, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from sedona_gpuspatial import _build, capi
    _build.build()
    return capi.lib()


def test_header_declarations_found():
    names = declared_functions()
    assert "GpuSpatialRuntimeCreate" in names and "SpjJoinProbeDevice" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lib):
    from sedona_gpuspatial import capi
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(capi.EXPORTS) <= set(declared_functions())


def test_version_string(lib):
    assert b"sm_103a" in lib.SpjVersion()


def test_runtime_init_fails_cleanly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sedona_gpuspatial import capi
    rt = capi.GpuSpatialRuntime()
    lib.GpuSpatialRuntimeCreate(C.byref(rt))
    cfg = capi.GpuSpatialRuntimeConfig(b"", 0, True, 0)
    rc = rt.init(C.byref(rt), C.byref(cfg))
    assert rc != 0
    assert len(rt.get_last_error(C.byref(rt))) > 0
    rt.release(C.byref(rt))


def test_object_create_rejects_uninitialized_runtime(lib):
    from sedona_gpuspatial import capi
    rt = capi.GpuSpatialRuntime()
    lib.GpuSpatialRuntimeCreate(C.byref(rt))
    idx = capi.SedonaFloatIndex2D()
    cfg = capi.GpuSpatialIndexConfig(C.pointer(rt), 1)
    assert lib.GpuSpatialIndexFloat2DCreate(C.byref(idx), C.byref(cfg)) != 0
    ref = capi.SedonaSpatialRefiner()
    rcfg = capi.GpuSpatialRefinerConfig(C.pointer(rt), 1, False, 1)
    assert lib.GpuSpatialRefinerCreate(C.byref(ref), C.byref(rcfg)) != 0
    rt.release(C.byref(rt))


def test_struct_layouts_match_reference_abi():
    """Sizes of the function-pointer structs as laid out by the reference
    header (c/sedona-libgpuspatial/libgpuspatial/include/gpuspatial/gpuspatial_c.h)."""
    from sedona_gpuspatial import capi
    p = C.sizeof(C.c_void_p)
    assert C.sizeof(capi.GpuSpatialRuntime) == 4 * p
    assert C.sizeof(capi.SedonaFloatIndex2D) == 10 * p
    assert C.sizeof(capi.SedonaSpatialRefiner) == 8 * p
    # const char*, int, bool (+3 padding), int; rounded up to pointer alignment
    assert C.sizeof(capi.GpuSpatialRuntimeConfig) == (p + 12 + p - 1) // p * p
    assert C.sizeof(capi.SpjJoinConfig) == p + 4 * 4
    # 5 u64, 4 u32, 5 f64, u64 ranges, 3 f64, 2 u32 windows, u64 launches
    assert C.sizeof(capi.SpjLearnedStats) == 5 * 8 + 4 * 4 + 5 * 8 + 8 + 3 * 8 + 2 * 4 + 8
    assert C.sizeof(capi.GpuSpatialRefinerConfig) == p + 4 + 1 + 3 + 4 + (4 if p == 8 else 0)


def test_option_keys_documented():
    """Every execution option SpjJoinSetOption accepts is documented in the
    public header, and vice versa."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = open(os.path.join(root, "sedona-db_gb300", "csrc", "capi.cu")).read()
    body = src[src.index("SpjJoinSetOption"):]
    body = body[:body.index("\n}\n")]
    accepted = set(re.findall(r'k == "([a-z_]+)"', body))
    hdr = open(os.path.join(root, "include", "spj_gb300.h")).read()
    block = hdr[hdr.index("Execution options"):hdr.index("int SpjJoinSetOption")]
    documented = set(re.findall(r'^ \*   "([a-z_]+)"', block, re.M))
    assert accepted, "no option keys found"
    assert accepted == documented, (accepted ^ documented)


def test_rust_bindings_name_declared_functions(lib):
    """Every function the Rust bindings (sedona-db_gb300/rust/spj_sys.rs)
    declare is declared in include/spj_gb300.h and exported by the library,
    and every #[repr(C)] struct they mirror has the header's field names in
    the header's order."""
    src = open(os.path.join(ROOT, "sedona-db_gb300", "rust", "spj_sys.rs")).read()
    rust_fns = sorted(set(re.findall(r"pub fn (Spj\w+)\s*\(", src)))
    assert len(rust_fns) > 20
    declared = set(declared_functions())
    missing = [f for f in rust_fns if f not in declared]
    assert not missing, missing
    for f in rust_fns:
        getattr(lib, f)
    hdr = open(os.path.join(ROOT, "include", "spj_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    for name, body in re.findall(
            r"#\[repr\(C\)\]\n(?:#\[derive\([^)]*\)\]\n)?pub struct (Spj\w+) \{(.*?)\n\}", src,
            flags=re.S):
        if "_private" in body:
            continue
        rust_fields = re.findall(r"pub (\w+):", body)
        m = re.search(r"struct " + name + r" \{(.*?)\};", hdr, flags=re.S)
        assert m, name
        c_fields = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            # "uint32_t partitions, passes" declares two fields
            head, *rest = [p.strip() for p in decl.split(",")]
            c_fields.append(re.findall(r"\w+", head)[-1])
            c_fields.extend(rest)
        assert rust_fields == c_fields, (name, rust_fields, c_fields)
