"""Failure detection of the tensor-core kernel without a GPU fault: every
mbarrier wait of tc_track_kernel gives up after one second, records the
failure in the device error flag and leaves (copies drained, tensor memory
freed).  A test hook withholds the kernel's weight loads, so the MMA
thread's weight wait runs out; the find must report Internal, and the next
find on the same context must be correct again."""
import ctypes as C
import json
import time
from pathlib import Path

import pytest

from golden.cases import CASES, make_inputs
from test_gpu_parity import assert_same_matches, gpu_find, gpu_model

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).parent / "golden" / "golden.json").read_text())["cases"]


@pytest.fixture(scope="module")
def mg():
    import mvkit_gb300
    from mvkit_gb300 import build
    build.build()
    mvkit_gb300.load()
    return mvkit_gb300


def test_tensor_core_wait_runs_out_and_context_recovers(mg):
    case = CASES["rot3_all"]
    wl, mask = make_inputs(case)
    model = gpu_model(mg, case, wl, mask)
    lib = mg.load()
    lib.mvg_test_withhold_tensor_weights.argtypes = [C.c_int32]
    lib.mvg_test_withhold_tensor_weights.restype = C.c_int32
    mg.set_correlation_path("tensor")
    assert lib.mvg_test_withhold_tensor_weights(1) == 0
    try:
        t0 = time.perf_counter()
        with pytest.raises(mg.MvError) as err:
            gpu_find(mg, model, wl.image, case)
        elapsed = time.perf_counter() - t0
    finally:
        assert lib.mvg_test_withhold_tensor_weights(0) == 0
    assert err.value.status == -1000
    assert "wait ran out" in err.value.message
    assert elapsed < 60, elapsed
    # the context is intact: the same find now gives the reference's matches
    assert_same_matches(gpu_find(mg, model, wl.image, case), GOLDEN["rot3_all"]["matches"], "after recovery")
