"""Host buffers of gb_upload / gb_download: pinned host memory (torch's
pinned tensors through the raw-pointer entry points, as bench.py's e2e line
uses them) and pageable numpy arrays must give the same state bit for bit,
through a few RK4 steps with a download and upload between them."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_pinned_and_pageable_host_buffers_agree():
    import torch

    import vipp_gb300
    x, v = O.plummer_reference(20000, 0.01, 5)
    n = x.shape[0]
    out = []
    for pinned in (False, True):
        with vipp_gb300.Solver(p=4, s=32, eps=0.01, m=1.0 / n, precision="mixed") as s:
            if pinned:
                xh = torch.from_numpy(x.copy()).pin_memory()
                vh = torch.from_numpy(v.copy()).pin_memory()
                s.upload_ptr(xh.data_ptr(), vh.data_ptr(), n)
                for _ in range(3):
                    s.solve(1e-3)
                    s.download_ptr(xh.data_ptr(), vh.data_ptr())
                    s.upload_ptr(xh.data_ptr(), vh.data_ptr(), n)
                out.append((xh.numpy().copy(), vh.numpy().copy()))
            else:
                s.preprocess(x, v)
                for _ in range(3):
                    s.solve(1e-3)
                    xs, vs = s.postprocess()
                    s.preprocess(xs, vs)
                out.append(s.postprocess())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert not np.array_equal(out[0][0], x)
