"""Differentiable image chains: torch.autograd.Function over the adjoint kernels.

    y = pipeline(x, [("rotate", theta), ("gaussian", sigma),
                     ("adjust_gamma", gamma), ("rgb2grey",)])
    (y * W).sum().backward()      # grads for x, theta, sigma, gamma

x is a float32 CUDA tensor of shape (B, H, W, C) (channels last, C in 1, 3, 4)
or (B, C, H, W) with channels_first=True.  Each op parameter is a python
float (same for every image) or a tensor of shape (B,) (per image; may
require grad).  adjust_gamma takes (gamma[, gain]), colorize (r, g, b).

Forward runs the fused batch path (mpk_chain_forward_saved) and, when a
backward will follow, keeps the intermediates the fused plan writes anyway
(the inputs of its later segments).  Backward (mpk_chain_backward_saved)
reads those, recomputes the other intermediates it needs image chunk by
image chunk (bounded scratch) and runs the adjoints in reverse -- one pass for each run of pointwise ops
(with their parameter gradients), blur(g) and, when sigma requires grad, two
derivative-tap dot passes for gaussian (d sigma), the exact transpose of the bilinear gather plus
d theta for rotate, and the inverse permutation for transpose / fliplr.
Parameter gradients accumulate in FP64.
"""
from __future__ import annotations

import ctypes as C
import weakref

import torch

from . import _abi

# name -> (MPOpCode, number of parameters)
_OPS = {
    "rgb2grey": (_abi.OP_RGB2GREY, 0), "rgb2gray": (_abi.OP_RGB2GREY, 0),
    "transpose": (_abi.OP_TRANSPOSE, 0), "fliplr": (_abi.OP_FLIPLR, 0),
    "gaussian": (_abi.OP_GAUSSIAN, 1), "rotate": (_abi.OP_ROTATE, 1),
    "brightness": (_abi.OP_BRIGHTNESS, 1), "adjust_gamma": (_abi.OP_ADJUST_GAMMA, 2),
    "colorize": (_abi.OP_COLORIZE, 3),
}
_DEFAULTS = {"adjust_gamma": (None, 1.0)}
# pointwise op codes (a run of them is one adjoint pass)
_PW = (_abi.OP_RGB2GREY, _abi.OP_BRIGHTNESS, _abi.OP_ADJUST_GAMMA, _abi.OP_COLORIZE)

_L = None


def _lib():
    global _L
    if _L is None:
        L = _abi.lib()
        L.mpk_chain_shape.restype = C.c_int
        L.mpk_chain_shape.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.mpk_chain_forward.restype = C.c_int
        L.mpk_chain_forward.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.mpk_chain_backward_masked.restype = C.c_int
        L.mpk_chain_backward_masked.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_void_p, C.c_void_p,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int),
                                                C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _L = L
    return _L


def _opcodes(names):
    arr = (C.c_int * max(1, len(names)))()
    for i, n in enumerate(names):
        arr[i] = _OPS[n][0]
    return arr


# Host tables of per-image parameters, reused while the device parameter
# tensors are the same live objects with unchanged version counters and the
# host parameters (python floats, CPU tensors) have the same values: the
# planner needs the values on the host (taps, rotation constants,
# footprints), and reading device tensors synchronises the device, so a
# forward whose parameters have not been written since the last one queues
# its launches without waiting for the previous step.  (Writes through
# `.data` bypass the version counter; write parameters in place under
# torch.no_grad(), as optimisers do.)
_PCACHE = []
_PCACHE_MAX = 8


def _param_table(B, nops, slots, ptensors):
    sig, dev_t = [], []
    for t in ptensors:
        if t.device.type == "cpu":
            sig.append(tuple(t.detach().reshape(-1).tolist()))
        else:
            sig.append(t._version)
            dev_t.append(t)
    key = (B, nops, tuple(slots), tuple(sig))
    for k, refs, P in _PCACHE:
        if k == key and len(refs) == len(dev_t) and all(r() is t for r, t in zip(refs, dev_t)):
            return P
    P = torch.zeros((B, max(1, nops), 3), dtype=torch.float64)
    cols = {}
    dev = [i for i, t in enumerate(ptensors) if t.device.type != "cpu"]
    if dev:
        # one copy for all device parameters (one synchronisation)
        flat = torch.cat([ptensors[i].detach().to(torch.float64).reshape(-1).expand(B) for i in dev]).cpu()
        for n, i in enumerate(dev):
            cols[i] = flat[n * B:(n + 1) * B]
    for i, t in enumerate(ptensors):
        if i not in cols:
            cols[i] = t.detach().to(torch.float64).reshape(-1).expand(B)
    for i, (k, j) in enumerate(slots):
        P[:, k, j] = cols[i]
    if len(_PCACHE) >= _PCACHE_MAX:
        _PCACHE.pop(0)
    _PCACHE.append((key, [weakref.ref(t) for t in dev_t], P))
    return P


class _ChainFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, names, slots, *ptensors):
        B, H, W, Cc = x.shape
        nops = len(names)
        # host table of explicit per-image parameters [B][nops][3]
        P = _param_table(B, nops, slots, ptensors)
        ops = _opcodes(names)
        L = _lib()
        ho, wo, co = C.c_int(), C.c_int(), C.c_int()
        _abi.check(L.mpk_chain_shape(ops, nops, H, W, Cc, C.byref(ho), C.byref(wo), C.byref(co)))
        y = torch.empty((B, ho.value, wo.value, co.value), device=x.device, dtype=torch.float32)
        stream = torch.cuda.current_stream(x.device).cuda_stream
        # with a backward to come, the forward keeps the intermediates it
        # writes anyway (segment boundaries) so that the backward does not
        # recompute them
        saved = None
        if any(ctx.needs_input_grad):
            cnt, nbytes = C.c_int(), C.c_size_t()
            _abi.check(L.mpk_chain_saved_layout(ops, nops, B, H, W, Cc, C.byref(cnt), None, None,
                                                C.byref(nbytes)))
            if nbytes.value:
                saved = torch.empty(nbytes.value, dtype=torch.uint8, device=x.device)
        _abi.check(L.mpk_chain_forward_saved(ops, nops, P.data_ptr(), x.data_ptr(), y.data_ptr(),
                                             saved.data_ptr() if saved is not None else None,
                                             B, H, W, Cc, stream))
        ctx.saved_inter = saved
        # a chain ending in a lone brightness back-propagates it from y
        ctx.y_used = nops >= 1 and names[-1] == "brightness" and (nops == 1 or _OPS[names[-2]][0] not in _PW)
        if ctx.y_used:
            ctx.save_for_backward(x, y)
        else:
            ctx.save_for_backward(x)
        ctx.P, ctx.names, ctx.slots, ctx.nparams = P, names, slots, len(ptensors)
        ctx.pshapes = [(t.shape, t.dtype, t.device) for t in ptensors]
        return y

    @staticmethod
    def backward(ctx, gy):
        x = ctx.saved_tensors[0]
        y = ctx.saved_tensors[1] if ctx.y_used else None
        B, H, W, Cc = x.shape
        gy = gy.contiguous()
        dx = torch.empty_like(x)
        nops = len(ctx.names)
        dP = torch.zeros((B, max(1, nops), 3), dtype=torch.float64, device=x.device)
        L = _lib()
        stream = torch.cuda.current_stream(x.device).cuda_stream
        # ops whose parameters want a gradient; the others skip their parameter passes
        mask = (C.c_int * max(1, nops))()
        for i, (k, _) in enumerate(ctx.slots):
            if ctx.needs_input_grad[3 + i]:
                mask[k] = 1
        sv = ctx.saved_inter
        _abi.check(L.mpk_chain_backward_saved(_opcodes(ctx.names), nops, ctx.P.data_ptr(), x.data_ptr(),
                                              sv.data_ptr() if sv is not None else None,
                                              y.data_ptr() if y is not None else None,
                                              gy.data_ptr(), dx.data_ptr(), dP.data_ptr(), mask,
                                              B, H, W, Cc, stream))
        ctx.saved_inter = None
        grads = []
        for i, ((k, j), (shape, dtype, dev)) in enumerate(zip(ctx.slots, ctx.pshapes)):
            if not ctx.needs_input_grad[3 + i]:
                # no gradient wanted (e.g. a constant python float): none is
                # formed, and none is copied to a host tensor
                grads.append(None)
                continue
            g = dP[:, k, j]
            g = g.sum().reshape(shape) if len(shape) == 0 or shape.numel() == 1 and B != 1 else g.reshape(shape)
            grads.append(g.to(device=dev, dtype=dtype))
        return (dx, None, None) + tuple(grads)


def pipeline(x: torch.Tensor, ops, channels_first: bool = False) -> torch.Tensor:
    """Apply a differentiable chain of image ops to a batch (see module doc).

    Returns (B, Ho, Wo, Co) float32 (channels last; (B, Co, Ho, Wo) when
    channels_first); a single output channel is squeezed: (B, Ho, Wo)."""
    if not x.is_cuda or x.dtype != torch.float32 or x.dim() != 4:
        raise TypeError("pipeline expects a 4-D float32 CUDA tensor")
    if channels_first:
        x = x.permute(0, 2, 3, 1)
    x = x.contiguous()
    B = x.shape[0]
    names, slots, ptensors = [], [], []
    for k, spec in enumerate(ops):
        name, args = spec[0], list(spec[1:])
        if name not in _OPS:
            raise ValueError("unknown op %r" % name)
        nparam = _OPS[name][1]
        dflt = _DEFAULTS.get(name, ())
        while len(args) < nparam and len(dflt) > len(args) and dflt[len(args)] is not None:
            args.append(dflt[len(args)])
        if len(args) != nparam:
            raise ValueError("%s takes %d parameter(s)" % (name, nparam))
        names.append(name)
        for j, a in enumerate(args):
            t = a if torch.is_tensor(a) else torch.tensor(float(a), dtype=torch.float64)
            if t.numel() not in (1, B):
                raise ValueError("parameter %d of %s must be a scalar or have %d entries" % (j, name, B))
            slots.append((k, j))
            ptensors.append(t)
    y = _ChainFn.apply(x, tuple(names), tuple(slots), *ptensors)
    if channels_first:
        y = y.permute(0, 3, 1, 2)
        return y[:, 0] if y.shape[1] == 1 else y
    return y[..., 0] if y.shape[-1] == 1 else y
