"""Thin ctypes wrappers over the surrogate's CUDA kernels (include/excalibur_mlp.h).

Every function takes device tensors (torch is only the allocator and the
stream) and launches on the current CUDA stream; nothing here computes on the
host. BF16 tensors are torch.bfloat16.
"""
from __future__ import annotations

import ctypes as C

from .. import _native as N

EPI = {"f32": N.EPI_F32, "bias_silu": N.EPI_BIAS_SILU, "dsilu": N.EPI_DSILU, "splitk": N.EPI_SPLITK}


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(t):
    import torch

    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _as3(t):
    return t if t.dim() == 3 else t.unsqueeze(0)


def gemm(a, b, *, epilogue="f32", bias=None, z_in=None, c=None, c2=None, ct=None, k_splits=1):
    """epilogue(A . B^T): a [E, M, K] bf16, b [E, N, K] bf16 (a 2-D operand is shared by
    every member: batch stride 0); outputs preallocated and contiguous:

    c:  f32 [E, M, N] ("f32"), f32 [E, splits, M, N] ("splitk"), bf16 [E, M, N] (others);
    c2: bf16 [E, M, N] (silu output); ct: bf16 [E, N, ldt] transposed output."""
    import torch

    M, K = a.shape[-2:]
    Nn, Kb = b.shape[-2:]
    E = max(a.shape[0] if a.dim() == 3 else 1, b.shape[0] if b.dim() == 3 else 1)
    if Kb != K or (a.dim() == 3 and a.shape[0] != E) or (b.dim() == 3 and b.shape[0] != E):
        raise ValueError("gemm: a [E,M,K] and b [E,N,K] must agree")
    for t in (a, b, c, c2, ct, z_in):
        if t is not None and not t.is_contiguous():
            raise ValueError("gemm: operands and outputs must be contiguous")
    if a.dtype != torch.bfloat16 or b.dtype != torch.bfloat16:
        raise TypeError("gemm: a and b must be bfloat16")
    g = N.ExcGemm()
    g.a, g.b = a.data_ptr(), b.data_ptr()
    g.m, g.n, g.k = M, Nn, K
    g.stride_a = M * K if a.dim() == 3 else 0
    g.stride_b = Nn * K if b.dim() == 3 else 0
    g.n_batch = E
    g.epilogue = EPI[epilogue]
    g.k_splits = int(k_splits)
    g.bias = bias.data_ptr() if bias is not None else None
    g.z_in = z_in.data_ptr() if z_in is not None else None
    g.c = c.data_ptr() if c is not None else None
    g.c2 = c2.data_ptr() if c2 is not None else None
    g.ct = ct.data_ptr() if ct is not None else None
    g.stride_c = M * Nn
    if ct is not None:
        g.ldt = ct.shape[-1]
        g.stride_ct = ct.shape[-2] * ct.shape[-1]
    lib = N.load()
    N.check(lib.exc_gemm_bf16(C.byref(g), _stream(a)), "exc_gemm_bf16")


def features(dirs, n_pad, n_freq, center, scale, out):
    """Fourier features of [n, 2] float64 (theta, phi) directions into out [n_pad, 4 n_freq] bf16."""
    lib = N.load()
    c2 = (C.c_double * 2)(*[float(v) for v in center])
    s2 = (C.c_double * 2)(*[float(v) for v in scale])
    N.check(lib.exc_mlp_features(_p(dirs), dirs.shape[0], n_pad, n_freq, c2, s2, _p(out), _stream(out)),
            "exc_mlp_features")


def infer(x, w, b, w_head, b_head, y):
    """The ensemble's forward pass in one launch (exc_mlp_infer): x [m, 256] bf16 features (m a
    multiple of 128), w [depth, E, 256, 256] bf16, b [depth, E, 256] f32, w_head [E, n_out, 256]
    f32, b_head [E, n_out] f32 -> y [E, m, n_out] f32 (preallocated)."""
    import torch

    for t in (x, w, b, w_head, b_head, y):
        if not t.is_contiguous():
            raise ValueError("infer: operands and output must be contiguous")
    if x.dtype != torch.bfloat16 or w.dtype != torch.bfloat16:
        raise TypeError("infer: x and w must be bfloat16")
    depth, E = w.shape[0], w.shape[1]
    a = N.ExcMlpInfer()
    a.x, a.w, a.b = x.data_ptr(), w.data_ptr(), b.data_ptr()
    a.w_head, a.b_head, a.y = w_head.data_ptr(), b_head.data_ptr(), y.data_ptr()
    a.m, a.width, a.n_members, a.n_out, a.depth = x.shape[0], x.shape[1], E, w_head.shape[1], depth
    N.check(N.load().exc_mlp_infer(C.byref(a), _stream(x)), "exc_mlp_infer")


def head(h, w, b, *, y=None, targets=None, z=None, dh=None, dht=None, dw=None, db=None, loss=None):
    """Linear head over h [E, M, 256] bf16 with w [E, n_out, 256] f32, b [E, n_out] f32."""
    E, M, width = h.shape
    n_out = w.shape[1]
    ldt = dht.shape[2] if dht is not None else 0
    lib = N.load()
    N.check(lib.exc_mlp_head(_p(h), M, width, n_out, E, _p(w), _p(b), _p(y), _p(targets), _p(z), _p(dh), _p(dht),
                             ldt, _p(dw), _p(db), _p(loss), _stream(h)), "exc_mlp_head")


def reduce_splits(part, out):
    """part [E, S, R, C] f32 -> out [E, R, C] (sum over S)."""
    E, S = part.shape[0], part.shape[1]
    rc = part[0, 0].numel()
    lib = N.load()
    N.check(lib.exc_mlp_reduce_splits(_p(part), E, S, rc, _p(out), _stream(part)), "exc_mlp_reduce_splits")


def row_sums(x, m, out):
    """Row sums of x [R, ld] bf16 over the first m columns -> out [R] f32."""
    rows, ld = x.shape[-2] * (x.shape[0] if x.dim() == 3 else 1), x.shape[-1]
    lib = N.load()
    N.check(lib.exc_mlp_row_sums(_p(x), rows, m, ld, _p(out), _stream(x)), "exc_mlp_row_sums")


def adam(p, g, m1, m2, *, lr, beta1, beta2, eps, t, p_bf16=None, pt_bf16=None, shape=None):
    rows, cols = shape if shape is not None else (0, 0)
    lib = N.load()
    N.check(lib.exc_mlp_adam(_p(p), _p(g), _p(m1), _p(m2), p.numel(), lr, beta1, beta2, eps, t, _p(p_bf16),
                             _p(pt_bf16), rows, cols, _stream(p)), "exc_mlp_adam")


def adam_multi(tensors, sched, *, beta1, beta2, eps):
    """One Adam step over every (p, g, m1, m2, p_bf16, pt_bf16, shape) in `tensors` in a single
    launch, {lr, 1/(1-beta1^t), 1/(1-beta2^t)} read from the float32 device tensor `sched`.
    """
    arr = (N.ExcAdamTensor * len(tensors))()
    for k, (p, g, m1, m2, pb, pt, shape) in enumerate(tensors):
        a = arr[k]
        a.p, a.grad, a.m1, a.m2 = p.data_ptr(), g.data_ptr(), m1.data_ptr(), m2.data_ptr()
        a.n = p.numel()
        a.p_bf16 = pb.data_ptr() if pb is not None else None
        a.pt_bf16 = pt.data_ptr() if pt is not None else None
        a.rows, a.cols = (shape if shape is not None else (0, 0))
    lib = N.load()
    N.check(lib.exc_mlp_adam_multi(arr, len(tensors), _p(sched), beta1, beta2, eps, _stream(sched)),
            "exc_mlp_adam_multi")


def error_count() -> int:
    v = C.c_uint32(0)
    N.check(N.load().exc_mlp_error_count(C.byref(v)), "exc_mlp_error_count")
    return int(v.value)
