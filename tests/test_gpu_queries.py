"""The compiled query (horsepower_gb300/queries/join_group.c) issues the same
builtin calls as the Python statement sequence (plans.join_group) and gives
the same bits, at a small size and at the benchmark's full size."""
import numpy as np
import pytest

from horsepower_gb300 import batch as B
from horsepower_gb300 import data as D
from horsepower_gb300 import plans as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import horsepower_gb300
    L = horsepower_gb300.load()
    assert P.compiled_queries(L) is not None, "libhgpu_queries.so missing"
    return L


@pytest.mark.parametrize("fact,dim,window", [(200_000, 50_000, (D.WIN_LO, D.WIN_HI)),
                                             (59_986_052, 15_000_000, (D.WIN_LO, D.WIN_HI)),
                                             (1_000_000, 250_000, (D.WIN_LO, D.WIN_LO + 30))])
def test_compiled_query_matches_statements(gpu, fact, dim, window):
    d, f = B.synth_tables(gpu, 77, fact, dim)
    mark = gpu.lib.getHeapOffset()
    a = [gpu.to_py(r) for r in P.join_group(gpu, d, f, *window)]
    b = [gpu.to_py(r) for r in P.join_group_compiled(gpu, d, f, *window)]
    gpu.lib.setHeapOffset(mark)
    assert len(a) == len(b) == 6
    for x, y in zip(a, b):
        x, y = np.atleast_1d(x), np.atleast_1d(y)
        assert x.dtype == y.dtype and x.tobytes() == y.tobytes()
    gpu.free_inputs()
