"""The packed (two-lane) FP32 arithmetic of the a-trous passes against the
scalar arithmetic, bit for bit: sgi_lane_selftest evaluates the packed
operations (also on exact rounding ties), exp over its whole range, x^128, a
pair of tap weights and their accumulation both ways on a million hashed
operand sets.
"""
import ctypes as C

import numpy as np
import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from stratusgfx_gb300 import abi  # noqa: E402

NAMES = ["add", "mul", "fma", "mul_tie", "add_tie", "fma_tie", "exp", "pow128", "atrous_weight2",
         "atrous_accumulate", "fma_subnormal_to_zero", "fma_subnormal_to_sum"]


def test_packed_lanes_equal_scalar_shading():
    lib = abi.load()
    counts = (C.c_uint32 * abi.SGI_LANE_CHECKS)()
    first = (C.c_float * (abi.SGI_LANE_CHECKS * 16))()
    assert lib.sgi_lane_selftest(1 << 20, counts, first) == abi.SGI_OK
    rec = np.frombuffer(first, np.float32).reshape(abi.SGI_LANE_CHECKS, 16)
    bad = [f"{NAMES[k]}: {int(counts[k])} threads; first: " + " ".join(f"{v:.9g}" for v in rec[k])
           for k in range(abi.SGI_LANE_CHECKS) if counts[k]]
    if bad:
        pytest.fail("\n".join(bad))
