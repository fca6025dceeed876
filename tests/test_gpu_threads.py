"""Host threads calling the library at once: the GPU entry points are serialised per
device inside the library (ctypes releases the interpreter lock around each call, so
the calls really overlap on the host). Four threads voxelize different fixtures, each
several times, in both precisions, and every result equals the sequential one bit for
bit."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIXTURES = ("shsphere64_r30p1", "icosphere_s3_r58p3", "cube4_r16p1", "uvsphere16_r20p1")
OUTS = 1 | 2  # occupancy + float distance


def _run(cm, g, precision):
    plc = cm.PLC.from_arrays(g["points"], g["triangles"])
    kw = dict(outputs=OUTS, precision=precision)
    if "resolution" in g:
        kw.update(resolution=int(g["resolution"]), pad=int(g["pad"]))
    else:
        kw.update(grid=(g["corner"], g["spacing"], g["dims"]))
    r = cm.voxelize_ex(plc, **kw)
    return np.array(r.occupancy), np.array(r.sdf32)


@pytest.mark.parametrize("precision", [0, 1])
def test_threads_get_the_sequential_results(cm, golden, precision):
    gs = [golden(n) for n in FIXTURES]
    want = [_run(cm, g, precision) for g in gs]
    got, errors = {}, []

    def worker(k):
        try:
            for rep in range(3):
                got[(k, rep)] = _run(cm, gs[k], precision)
        except Exception as e:  # reported below, on the main thread
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(len(gs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not errors, errors
    assert len(got) == 3 * len(gs)
    for (k, _), (occ, sdf) in got.items():
        assert np.array_equal(occ, want[k][0])
        assert np.array_equal(sdf.view(np.uint32), want[k][1].view(np.uint32))
