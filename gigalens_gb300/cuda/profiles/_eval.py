"""Elementwise evaluation of one profile through ``gl_profile_eval``."""
import torch

from ... import _native as N


def _dev():
    if not torch.cuda.is_available():
        raise RuntimeError("gigalens_gb300.cuda needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


def as_cuda(v, dev):
    return torch.as_tensor(v, dtype=torch.float32, device=dev)


def evaluate(kind, x, y, params, niter=0):
    """Evaluate profile ``kind`` at (x, y) with broadcastable parameters.

    Returns one tensor (light) or a pair (deflection) shaped like the broadcast
    of x, y and the parameters.
    """
    dev = _dev()
    names = N.CANONICAL_PARAMS[kind]
    tensors = [as_cuda(x, dev), as_cuda(y, dev)] + [as_cuda(params[k], dev) for k in names]
    shape = torch.broadcast_shapes(*[t.shape for t in tensors])
    xs, ys = (t.expand(shape).reshape(-1).contiguous() for t in tensors[:2])
    n = xs.numel()
    prm = torch.stack([t.expand(shape).reshape(-1) for t in tensors[2:]], dim=0).contiguous()
    out0 = torch.empty(n, dtype=torch.float32, device=dev)
    mass = kind in ("EPL", "SHEAR", "SIS", "SIE", "TNFW")
    out1 = torch.empty(n, dtype=torch.float32, device=dev) if mass else None
    kt = None
    stream = N.stream_ptr()
    if kind == "EPL":
        # the reference's batch-coupled term count, over the parameter tensors
        e1 = as_cuda(params["e1"], dev).reshape(-1).contiguous()
        e2 = as_cuda(params["e2"], dev).reshape(-1).contiguous()
        e1, e2 = torch.broadcast_tensors(e1, e2)
        e1, e2 = e1.contiguous(), e2.contiguous()
        kt = torch.empty(1, dtype=torch.int32, device=dev)
        N.call("gl_epl_term_count", N.ptr(e1), N.ptr(e2), e1.numel(), int(niter), N.ptr(kt), stream)
    if n > 0:
        N.call("gl_profile_eval", N.PROFILE_TYPES[kind], N.ptr(xs), N.ptr(ys), n, N.ptr(prm), N.ptr(kt),
               N.ptr(out0), N.ptr(out1), stream)
    if mass:
        return out0.reshape(shape), out1.reshape(shape)
    return out0.reshape(shape)
