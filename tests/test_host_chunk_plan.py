"""The host-buffer step's chunk plan (pf_rstep_host cuts the cells into
chunks whose copies overlap the compute): up to 2^18 cells one chunk, else a
tenth of the cells, the rest and a tenth; every chunk but the last starts on
a whole 64-cell group and the chunks cover the cells exactly once.  Host
logic only: the library loads without a GPU and the plan does no device
work."""
import ctypes as C

import pytest

from pfgpu import abi


@pytest.fixture(scope="module")
def plan():
    from pfgpu import build
    build.build()  # incremental: recompiles only changed translation units
    lib = abi.load()
    fn = lib.pf_internal_host_chunk_plan
    fn.restype = C.c_int32
    fn.argtypes = [C.c_int64, C.POINTER(C.c_int64)]

    def call(n):
        starts = (C.c_int64 * 4)()
        k = fn(n, starts)
        assert 1 <= k <= 3
        return [starts[i] for i in range(k + 1)]
    return call


@pytest.mark.parametrize("n", [1, 63, 64, 1000, 262143, 262144, 262145, 262207, 600000, 1_000_000,
                               1_048_576, 4_000_003, 10_000_000, 2 ** 31 + 5])
def test_chunks_cover_the_cells_aligned(plan, n):
    b = plan(n)
    assert b[0] == 0 and b[-1] == n
    assert all(lo < hi for lo, hi in zip(b, b[1:]))
    assert all(x % 64 == 0 for x in b[:-1])
    if n <= 2 ** 18:
        assert len(b) == 2
    else:
        assert len(b) == 4
        edge = -(-n // 10)
        assert edge <= b[1] < edge + 64                # the first chunk: a tenth, rounded up to 64
        assert 0 <= (n - b[2]) - b[1] < 64             # the last one: the same, plus the ragged end
        assert b[2] - b[1] > 7 * (n // 10)             # the rest in the middle


def test_bad_arguments(plan):
    lib = abi.load()
    assert lib.pf_internal_host_chunk_plan(-1, (C.c_int64 * 4)()) == -1
    assert lib.pf_internal_host_chunk_plan(10, None) == -1
