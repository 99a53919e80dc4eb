"""The C ABI without a GPU: the library loads, exports every function include/trans_gpu.h
declares, the ctypes mirror has the C compiler's layout, and option validation answers with
status codes before any device work."""
import ctypes as C
import os
import re
import subprocess

import pytest

from trans_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "trans_gpu.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(trans_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from trans_gb300 import native
    try:
        return native.load()
    except native.NativeUnavailable as e:      # no nvcc in this environment
        pytest.skip(str(e))


def test_every_declared_function_is_exported(lib):
    names = _declared()
    assert "trans_create" in names and "trans_iterate" in names
    for n in names:
        assert hasattr(lib, n), f"{n} declared in trans_gpu.h but not exported"
        assert n in abi.EXPORTED, f"{n} missing from trans_gb300.abi.EXPORTED"


def _c_layout(tmp_path):
    """sizeof/offsetof of the ABI structs as the C compiler lays them out."""
    fields = {
        "trans_params": [f for f, _ in abi.TransParams._fields_],
        "trans_conn": [f for f, _ in abi.TransConn._fields_],
        "trans_block": [f for f, _ in abi.TransBlock._fields_],
        "trans_norms": [f for f, _ in abi.TransNorms._fields_],
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for s, fs in fields.items():
        lines.append(f'printf("{s} sizeof %zu\\n", sizeof({s}));')
        for f in fs:
            lines.append(f'printf("{s} {f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-o", str(exe), str(src)])
    out = subprocess.check_output([str(exe)]).decode().split("\n")
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}


def test_struct_layout_matches_header(tmp_path):
    lay = _c_layout(tmp_path)
    for name, cls in (("trans_params", abi.TransParams), ("trans_conn", abi.TransConn),
                      ("trans_block", abi.TransBlock), ("trans_norms", abi.TransNorms)):
        assert lay[(name, "sizeof")] == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert lay[(name, f)] == getattr(cls, f).offset, (name, f)


def test_enums_match_header():
    src = open(HEADER).read()
    for i, f in enumerate(abi.FIELDS):
        m = re.search(r"TRANS_%s\s*=\s*(\d+)" % f, src)
        assert m and int(m.group(1)) == i, f
    for i, s in enumerate(abi.STAGES):
        m = re.search(r"TRANS_STAGE_%s\s*=\s*(\d+)" % s, src)
        assert m and int(m.group(1)) == i, s


def _params(**kw):
    from trans_gb300 import cases
    p = cases.channel_bump(25, 17, 6).params
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("bad", [dict(IF_RK=2), dict(IF_Precondition=2), dict(IF_Precondition=1, precision=1),
                                 dict(IF_Precondition=1, IF_RK=1), dict(Kind_RotMod=3), dict(Kind_Model=3),
                                 dict(Kind_Spatial=5), dict(Kind_Spatial=0), dict(Kind_Roe=4), dict(Kind_Hybrid=1),
                                 dict(IF_Euler=1),
                                 dict(precision=7)])
def test_unsupported_options_are_rejected(lib, bad):
    """Options outside the path answer TRANS_E_ARG from trans_create; no device memory is touched."""
    p = _params(**bad)
    blk = (abi.TransBlock * 1)()
    blk[0].ni = blk[0].nj = blk[0].nk = 8
    ctx = C.c_void_p()
    assert lib.trans_create(C.byref(p), 1, blk, C.byref(ctx)) == abi.TRANS_E_ARG
    assert not ctx.value


def test_non_finite_rotation_is_rejected(lib):
    """omega(1) is the frame's rotation about x; any finite value is accepted, NaN or inf is not."""
    p = _params()
    p.omega[0] = float("nan")
    blk = (abi.TransBlock * 1)()
    blk[0].ni = blk[0].nj = blk[0].nk = 8
    ctx = C.c_void_p()
    assert lib.trans_create(C.byref(p), 1, blk, C.byref(ctx)) == abi.TRANS_E_ARG
    assert not ctx.value


def test_null_arguments_are_rejected(lib):
    ctx = C.c_void_p()
    assert lib.trans_create(None, 1, None, C.byref(ctx)) == abi.TRANS_E_ARG
    assert lib.trans_iterate(None, 1, None) == abi.TRANS_E_ARG
    assert lib.trans_destroy(None) == abi.TRANS_OK      # like free(NULL)


def test_rotated_roe_is_fp64_only(lib):
    """The rotated Roe scheme (Kind_Roe = 2) runs in the FP64 path; the mixed path refuses it."""
    p = _params(Kind_Roe=2, precision=abi.TRANS_MIXED)
    blk = (abi.TransBlock * 1)()
    blk[0].ni = blk[0].nj = blk[0].nk = 8
    ctx = C.c_void_p()
    assert lib.trans_create(C.byref(p), 1, blk, C.byref(ctx)) == abi.TRANS_E_ARG


def test_conversion_check_validates_arguments_before_any_device_work(lib):
    """trans_check_conversions rejects a pattern count outside 1..2^32 or a NULL result array
    with TRANS_E_ARG and a message, before it touches the device (so this runs without one)."""
    bad = (C.c_longlong * 2)()
    assert lib.trans_check_conversions(0, 1, bad) == abi.TRANS_E_ARG
    assert lib.trans_check_conversions((1 << 32) + 1, 1, bad) == abi.TRANS_E_ARG
    assert lib.trans_check_conversions(16, 1, None) == abi.TRANS_E_ARG
    assert b"trans_check_conversions" in lib.trans_last_error(None)
