"""torch.autograd binding of the fused likelihood-and-gradient kernel.

``log_likelihood(gb, params, data, psd, **kw)`` returns logL (B,) as a torch
tensor that is differentiable with respect to ``params`` (9, B), or (14, B)
for ``GBGPUThirdBody``: the forward launch computes logL and its gradient
together (``gbx_waveform_ll_grad``), the backward multiplies the stored
gradient by the incoming one.
"""

import torch


class _LogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, gb, data, psd, kwargs):
        """Likelihood and its gradient in one fused launch; the gradient is kept for backward."""
        like, grad = gb._ll_grad_tensors(params.detach(), data, psd, **kwargs)
        ctx.save_for_backward(grad)
        return like

    @staticmethod
    def backward(ctx, g):
        """Chain rule: d like / d params scaled by the incoming gradient per binary."""
        (grad,) = ctx.saved_tensors
        return grad * g.to(grad.dtype)[None, :], None, None, None, None


def log_likelihood(gb, params, data, psd, **kwargs):
    """Differentiable logL of each binary; ``params`` is a (gb.NPARAMS, B) FP64 CUDA tensor."""
    return _LogLikelihood.apply(params, gb, data, psd, kwargs)
