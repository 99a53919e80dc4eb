"""The integer-pipe double <-> float conversions of the mixed-precision kernels
(trans_gb300/csrc/cvt.cuh) against the GPU's own conversions: bit-identical on 2^26 random
and edge-case patterns per seed (round to nearest even, signed zeros, the float range limits,
infinities, NaN)."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 20261204])
def test_conversions_match_hardware(gpu_lib, seed):
    bad = (C.c_longlong * 2)()
    rc = gpu_lib.trans_check_conversions(1 << 26, seed, bad)
    assert rc == 0, gpu_lib.trans_last_error(None)
    assert list(bad) == [0, 0], f"double->float mismatches {bad[0]}, float->double {bad[1]}"


def test_conversion_check_rejects_bad_arguments(gpu_lib):
    from trans_gb300 import abi
    bad = (C.c_longlong * 2)()
    assert gpu_lib.trans_check_conversions(0, 1, bad) == abi.TRANS_E_ARG
    assert gpu_lib.trans_check_conversions(16, 1, None) == abi.TRANS_E_ARG
