"""Failure detection without a GPU fault: a bounded device wait is made to
give up, and the call reports it while the context stays usable.

The radix sort of the tree build waits, per tile, for the digit counts that
earlier tiles publish (a decoupled look-back); every wait is bounded
(kSortSpinMax polls), and a wait that gives up sets kDevTimeout in the
evaluation's status word and reads the missing count from that tile's keys
instead, so the sort's output stays exact. VIPP_GB_SORT_WAIT_POLLS=0 (read at
gb_create / gb_set_config) makes every look-back give up at its first poll.
Nothing here hangs or faults: the fallback reads only the pass's own input.
"""
import numpy as np
import pytest

import oracle as O
from treecmp import canon_gpu, diff_trees

pytestmark = pytest.mark.gpu


def test_sort_wait_gives_up_is_reported_and_context_recovers(monkeypatch):
    import vipp_gb300
    x, v = O.plummer_reference(40000, 0.01, 3)  # 10 sort tiles per pass
    n = x.shape[0]
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n, precision="mixed") as s:
        s.preprocess(x, v)
        clean = s.accel()
        clean_tree = canon_gpu(s.tree_dump())
    monkeypatch.setenv("VIPP_GB_SORT_WAIT_POLLS", "0")
    with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n, precision="mixed") as s:
        s.preprocess(x, v)
        with pytest.raises(vipp_gb300.GB300Error) as ei:
            s.accel()
        assert ei.value.code == vipp_gb300.GB_ERR_CUDA and "gave up" in str(ei.value)
        # the sort stayed exact: the tree of the reported evaluation is the clean one
        assert diff_trees(canon_gpu(s.tree_dump()), clean_tree) == []
        # an RK4 step reports it too (through the step or the next sync)
        with pytest.raises(vipp_gb300.GB300Error):
            s.solve(1e-3)
            s.sync()
        # recovery: the normal limit again on the same context
        monkeypatch.delenv("VIPP_GB_SORT_WAIT_POLLS")
        s.set_config()
        s.preprocess(x, v)
        assert np.array_equal(s.accel(), clean)
        s.solve(1e-3)
        s.sync()
