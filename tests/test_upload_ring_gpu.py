"""GPU: plan tables reach the device through a page-locked ring that is
reused lap after lap.  Many batches are queued without waiting (each with
its own rotation angle and output buffers, more table bytes in total than
the 32 MB ring holds, so slots are handed out again while earlier copies
may still be queued); every sampled output must still be the oracle's for
its own angle."""
import ctypes as C

import numpy as np
import pytest

from millipyde_gb300 import _abi
from oracle import oracle as O

from helpers import TOL, maxabs

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_queued_batches_keep_their_own_tables(gpu):
    L = _abi.lib()
    n, h, w, calls = 256, 24, 20, 120          # 256 jobs x 1.5 KB per table: ~46 MB over all calls
    rng = np.random.default_rng(71)
    xs = rng.random((n, h, w, 3), dtype=np.float32)
    x = torch.from_numpy(xs.reshape(n, h, w * 3)).cuda()
    y = torch.full((calls, n, h, w * 3), float("nan"), device="cuda")
    ins = _abi.images([_abi.image(x[i].data_ptr(), h, w, 3, w * 12) for i in range(n)])
    angles = [-60.0 + 120.0 * c / (calls - 1) for c in range(calls)]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs_keep = []
    torch.cuda.synchronize()
    for c in range(calls):
        outs = _abi.images([_abi.image(y[c, i].data_ptr(), h, w, 3, w * 12) for i in range(n)])
        outs_keep.append(outs)
        _abi.check(L.mpk_pipeline_run(_abi.stages(_abi.stage("rotate", angles[c])), 1, ins, outs, n, 0, 0,
                                      stream))
    torch.cuda.synchronize()
    for c in (0, 1, 37, 59, 60, 61, 100, 118, 119):
        for i in (0, 101, 255):
            ref = O.run_ops(xs[i], [("rotate", angles[c])])
            got = y[c, i].cpu().numpy().reshape(h, w, 3)
            assert maxabs(got, ref) <= TOL, (c, i)
