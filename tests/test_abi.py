"""The C-ABI library loads, exports every entry point declared in include/*.h, and rejects bad
arguments on the host (no GPU work)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        names |= set(re.findall(r"^\s*(?:const\s+)?(?:long\s+long|\w+)\s*\*?\s*(cov3d_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "cov3d_plan_create" in names and "cov3d_covar_cost_grad" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(pkg._lib.exported_symbols()) == declared_symbols()


def test_host_side_validation(pkg):
    lib = pkg._lib.load()
    assert lib.cov3d_abi_version() == 1
    h = ctypes.c_void_p()
    assert lib.cov3d_plan_create(0, 1, 1e-6, None, ctypes.byref(h)) == pkg._lib.EINVAL
    assert "invalid plan size" in pkg._lib.last_error()
    opts = pkg._lib.Opts(kernel=7, upsample=2)
    assert lib.cov3d_plan_create(16, 1, 1e-6, ctypes.byref(opts), ctypes.byref(h)) == pkg._lib.EINVAL
    assert lib.cov3d_plan_destroy(None) == 0
    assert lib.cov3d_setpts(None, None, 1, 4, 48, 16, 0) == pkg._lib.EINVAL
    assert lib.cov3d_mean_accumulate(None, None, None, None, None, None, 0) == pkg._lib.EINVAL
    assert lib.cov3d_regularize_lhs(None, None, None) == pkg._lib.EINVAL
    assert lib.cov3d_mean_init(None, None, None, None, None) == pkg._lib.EINVAL
    assert lib.cov3d_circulant_symbol(None, None, None) == pkg._lib.EINVAL
    it, rr = ctypes.c_int(), ctypes.c_double()
    assert lib.cov3d_cg_solve(None, None, None, None, 1e-6, 10, 0, None, ctypes.byref(it), ctypes.byref(rr),
                              None) == pkg._lib.EINVAL
    assert "cg_solve" in pkg._lib.last_error()
    assert lib.cov3d_status_string(pkg._lib.ENOMEM) == b"out of device memory"
    try:
        pkg._lib.check(pkg._lib.EINVAL)
    except ValueError as e:
        assert "invalid argument" in str(e)
    else:
        raise AssertionError("check() did not raise")


def _header_text():
    text = "".join(open(h).read() for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))))
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def test_binding_matches_every_prototype(pkg):
    """The ctypes table (_lib._SIGNATURES) gives every prototype of the header the same number of
    arguments, so a parameter added on one side only fails here rather than on the GPU."""
    protos = re.findall(r"\b(cov3d_\w+)\s*\(([^;{}]*?)\)\s*;", _header_text(), flags=re.S)
    assert len(protos) >= 15
    sigs = pkg._lib._SIGNATURES
    for name, params in protos:
        p = params.strip()
        n = 0 if p in ("", "void") else p.count(",") + 1
        assert name in sigs, name
        assert len(sigs[name][1]) == n, (name, n, len(sigs[name][1]))


def test_binding_structs_match_the_header(pkg):
    """cov3d_opts and cov3d_cost_args: the same fields in the same order on both sides."""
    text = _header_text()
    for sname, cls in (("cov3d_opts", pkg._lib.Opts), ("cov3d_cost_args", pkg._lib.CostArgs)):
        m = re.search(r"typedef struct\s*\w*\s*\{([^{}]*)\}\s*" + sname + r"\s*;", text)
        assert m, sname
        fields = [re.findall(r"(\w+)\s*$", f.strip())[0] for f in m.group(1).split(";") if f.strip()]
        assert fields == [f[0] for f in cls._fields_], sname
