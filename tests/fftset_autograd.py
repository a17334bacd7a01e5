"""A torch.autograd.Function over the fftset C ABI, for the tests only.

ConvFn.apply(x, h, plan): y_b = fftset_fft_conv(x_b, fftset_fft_conv_get_kernel(h))
for a batch x [B, 2L] and taps h [2L] (CUDA float32). The backward pass is
the library's hand-written adjoint, fftset_fft_conv_adjoint_batch: grad_x by
the convolution with the conjugated kernel spectrum, grad_h by the batch sum
of cross-correlations. The product ships no autograd layer; this wrapper only
lets the tests drive the adjoint the way a training loop would.
"""
import torch


class ConvFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, h, plan):
        K = torch.empty_like(h)
        plan.conv_get_kernel(K, h)
        y = torch.empty_like(x)
        plan.conv_batch(y, x, K)
        ctx.save_for_backward(x, K)
        ctx.plan = plan
        return y

    @staticmethod
    def backward(ctx, gy):
        x, K = ctx.saved_tensors
        gy = gy.contiguous()
        dx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        dh = torch.empty(K.shape, device=K.device, dtype=K.dtype) if ctx.needs_input_grad[1] else None
        ctx.plan.conv_adjoint_batch(dx, dh, gy, x, K)
        return dx, dh, None
