"""Device-memory cap of an engine (isspa_engine_options.mem_cap).

* an engine is refused with ISSPA_ERR_NOMEM below the bytes it needs, and the
  smallest cap it is created under is found by bisection (to 16 bytes);
* at that cap the neighbour- and cell-list queries, whose temporary device
  buffers count against the cap, are refused with ISSPA_ERR_NOMEM;
* with the cap raised by exactly those temporary bytes they run and return
  what an uncapped engine returns;
* refused creations leave the process able to create engines.
"""
import numpy as np
import pytest

import isspa_gb300 as ig
from isspa_gb300 import abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system():
    return ig.synth.make_system(6, 22, 36.0, 20, seed=8, ff=ig.synth.forcefield(n_mc=20))


def _fits(s, cap):
    try:
        ig.Engine(s, mem_cap=cap).close()
        return True
    except ig.IsspaError as e:
        assert e.status == abi.ERR_NOMEM
        return False


def test_mem_cap_bounds_engine_and_list_queries(system):
    n = system.n_atoms
    assert not _fits(system, 4096)
    lo, hi = 4096, 1 << 30
    assert _fits(system, hi)
    while hi - lo > 16:
        mid = (lo + hi) // 2
        if _fits(system, mid):
            hi = mid
        else:
            lo = mid
    # hi - 16 < bytes held by the engine <= hi
    per = 64
    nl_tmp = 4 * (n * per + n)  # rows and counts, int32
    cl_tmp = 4 * n              # cell index per atom, int32
    eng = ig.Engine(system, mem_cap=hi)
    for query in (lambda: eng.neighbor_list(6.0, max_per_atom=per), lambda: eng.cell_list(9.0, (4, 4, 4))):
        with pytest.raises(ig.IsspaError) as e:
            query()
        assert e.value.status == abi.ERR_NOMEM
    eng.step(3)  # the refused queries left the engine usable
    assert eng.device_status() == 0
    eng.close()

    free = ig.Engine(system)
    rows_ref, counts_ref = free.neighbor_list(6.0, max_per_atom=per)
    cell_ref = free.cell_list(9.0, (4, 4, 4))
    free.close()
    a = ig.Engine(system, mem_cap=hi + nl_tmp)
    rows, counts = a.neighbor_list(6.0, max_per_atom=per)
    assert np.array_equal(counts, counts_ref)
    assert np.array_equal(rows, rows_ref)
    a.close()
    b = ig.Engine(system, mem_cap=hi + cl_tmp)
    assert np.array_equal(b.cell_list(9.0, (4, 4, 4)), cell_ref)
    b.close()
