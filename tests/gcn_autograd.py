"""Test-harness-only autograd wrapper of the library's SpMM forward and
backward kernels (the library itself exposes them through the C ABI):
  forward : Y = A(vals) @ H            (merge-path CSR SpMM)
  backward: dH = A^T @ dY and dvals[e] = <dY[row e], H[col e]>, fused in
            one pass over the cached transpose (gbs_spmm_backward)
Features (H, dY) are handed to the kernels in `feat_dtype` (FP32 or BF16);
accumulation and outputs are FP32."""
import torch

from spmm_eval_gb300 import ops


class SpMMFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vals, H, pattern, transpose, feat_dtype):
        Hk = H.detach().to(feat_dtype).contiguous()
        A = ops.CSR(pattern.rowptr, pattern.colind, vals.detach().contiguous(), pattern.nrows, pattern.ncols)
        Y = ops.csr_spmm(A, Hk)
        ctx.save_for_backward(vals, Hk)
        ctx.pattern, ctx.transpose, ctx.feat_dtype = pattern, transpose, feat_dtype
        return Y

    @staticmethod
    def backward(ctx, gY):
        vals, Hk = ctx.saved_tensors
        p, T = ctx.pattern, ctx.transpose
        Gk = gY.detach().to(ctx.feat_dtype).contiguous()
        # fused: dH = A^T dY and dvals = SDDMM(dY, H) in one pass over A^T
        dH, dvals = ops.spmm_backward(T, T.values(vals.detach().contiguous()), Gk, Hk)
        return dvals, dH, None, None, None


def gcn_layer(vals, X, W, pattern, transpose, feat_dtype=torch.float32):
    """Y = A_hat (X W); the dense X W product is torch's."""
    return SpMMFunction.apply(vals, X @ W, pattern, transpose, feat_dtype)
