"""HostStreamer: slices from pinned host memory through the parallel FBP
pipeline with overlapped copies give exactly the results of running each
slice alone (same kernels, same order on one compute stream)."""
import numpy as np
import pytest

from gpu_helpers import fp_op, par_op, ramp_op

pytestmark = pytest.mark.gpu


def test_streamed_equals_serial():
    import torch
    from ct_recon_extensions_gb300 import synthetic as syn
    from ct_recon_extensions_gb300.host_stream import HostStreamer
    g = syn.parallel_config_2()
    fp, ramp, bp = fp_op(g), ramp_op(g, g["na"], 0, dsd=-1.0), par_op(g)

    def serial(x):
        return bp.forward(ramp.forward(fp.forward(x)))

    def step(din, dout, s):
        with torch.cuda.stream(torch.cuda.ExternalStream(s)):
            dout.copy_(serial(din))

    rng = np.random.default_rng(5)
    n = 7
    ins = [torch.from_numpy(rng.random((g["ny"], g["nx"]), dtype=np.float32)).pin_memory() for _ in range(n)]
    outs = [torch.empty((g["ny"], g["nx"]), dtype=torch.float32).pin_memory() for _ in range(n)]
    for depth in (1, 2, 3):
        for o in outs:
            o.fill_(float("nan"))
        HostStreamer(step, (g["ny"], g["nx"]), (g["ny"], g["nx"]), "cuda", depth=depth).run(ins, outs)
        for x, o in zip(ins, outs):
            ref = serial(x.cuda()).cpu()
            assert torch.equal(o, ref)
