"""Batches of independent systems (gb_batch_*): every system of a batch step
must equal the same system stepped alone in its own context, bit for bit,
in both precisions and with either tensor-core M2L split; uneven sizes, an empty and a one-particle system, per-system
masses, and a system whose first step overflows its buffers (repeated alone)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def systems():
    out = []
    for k, n in enumerate([1500, 1, 0, 3000, 2048]):
        x, v = O.plummer_reference(n, 0.01, 10 + k) if n > 1 else (np.full((n, 3), 0.25), np.zeros((n, 3)))
        out.append((x * (0.5 + 0.3 * k), v / np.sqrt(0.5 + 0.3 * k)))
    return out


@pytest.mark.parametrize("precision,bf16", [("fp64", False), ("mixed", False), ("mixed", True)])
def test_batch_equals_separate_contexts(precision, bf16):
    import vipp_gb300
    flags = vipp_gb300.FLAG_M2L_BF16 if bf16 else 0
    sy = systems()
    sizes = [len(x) for x, _ in sy]
    masses = [1.0 / max(n, 1) for n in sizes]
    X = np.concatenate([x for x, _ in sy]) if sum(sizes) else np.zeros((0, 3))
    V = np.concatenate([v for _, v in sy])
    with vipp_gb300.Batch(sizes, p=5, s=16, eps=0.01, masses=masses, precision=precision, flags=flags) as b:
        b.upload(X, V)
        for dt in (1e-3, 1e-3, 2e-3):
            b.step(dt)
        xb, vb = b.download()
        a3 = b.system_accel(3)
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k, (x, v) in enumerate(sy):
        if len(x) == 0:
            continue
        with vipp_gb300.Solver(p=5, s=16, eps=0.01, m=masses[k], precision=precision, flags=flags) as s:
            s.preprocess(x, v)
            for dt in (1e-3, 1e-3, 2e-3):
                s.solve(dt)
            xs, vs = s.postprocess()
            if k == 3:
                assert np.array_equal(s.accel(), a3)
        assert np.array_equal(xb[off[k]:off[k + 1]], xs) and np.array_equal(vb[off[k]:off[k + 1]], vs)


def test_batch_system_overflow_is_repeated():
    import vipp_gb300
    x, v = O.plummer_reference(100_000, 0.01, 0)  # needs 3x the initial partial-sum slots at s = 256
    y, w = O.plummer_reference(4000, 0.01, 1)
    sizes = [len(y), len(x)]
    with vipp_gb300.Batch(sizes, p=4, s=256, eps=0.01, masses=[1 / len(y), 1 / len(x)], precision="mixed") as b:
        b.upload(np.concatenate([y, x]), np.concatenate([w, v]))
        b.step(1e-3)
        xb, vb = b.download()
    with vipp_gb300.Solver(p=4, s=256, eps=0.01, m=1 / len(x), precision="mixed") as s:
        s.preprocess(x, v)
        s.solve(1e-3)
        xs, vs = s.postprocess()
    assert np.array_equal(xb[len(y):], xs) and np.array_equal(vb[len(y):], vs)
