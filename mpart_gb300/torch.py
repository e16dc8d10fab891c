"""torch.autograd wrapper: the reference's MpartTorchAutograd and
TorchConditionalMapBase (bindings/python/package/torch_helpers.py:33-114,
bindings/python/package/torch.py:32-106), with the backward pass served by one
fused adjoint call instead of separate Gradient/CoeffGrad/LogDeterminant*Grad
calls followed by host-side sums."""
from __future__ import annotations

import torch


class MpartTorchAutograd(torch.autograd.Function):

    @staticmethod
    def forward(ctx, input, coeffs, f, return_logdet):
        ctx.save_for_backward(input, coeffs)
        ctx.f = f
        if coeffs is not None:
            c = coeffs.detach().to(device=input.device, dtype=torch.float64).contiguous()
            f.WrapCoeffs(c)
            ctx.c = c
        x = input.detach().to(torch.float64)
        out = torch.zeros(f.outputDim, x.shape[1], dtype=torch.float64, device=x.device)
        if return_logdet:
            ld = torch.zeros(x.shape[1], dtype=torch.float64, device=x.device)
            f.FusedForwardAdjointImpl(x, out_eval=out, out_logdet=ld)
            return out.to(input.dtype), ld.to(input.dtype)
        f.EvaluateImpl(x, out)
        return out.to(input.dtype)

    @staticmethod
    def backward(ctx, output_sens, logdet_sens=None):
        input, coeffs = ctx.saved_tensors
        f = ctx.f
        if coeffs is not None:
            f.WrapCoeffs(ctx.c)
        x = input.detach().to(torch.float64)
        sens = output_sens.detach().to(torch.float64).contiguous() if output_sens is not None else None
        lsens = logdet_sens.detach().to(torch.float64).contiguous() if logdet_sens is not None else None
        grad = None
        coeff_grad = None
        want_x = input.requires_grad
        want_c = coeffs is not None and coeffs.requires_grad
        if want_x:
            grad = torch.zeros(f.inputDim, x.shape[1], dtype=torch.float64, device=x.device)
        if want_c:
            coeff_grad = torch.zeros(f.numCoeffs, dtype=torch.float64, device=x.device)
        if want_x or want_c:
            f.FusedForwardAdjointImpl(x, sens=sens, logdet_sens=lsens, logdet_sens_scale=0.0,
                                      coeff_grad=coeff_grad, input_grad=grad)
        if grad is not None:
            grad = grad.to(input.dtype)
        if coeff_grad is not None:
            coeff_grad = coeff_grad.to(coeffs.dtype)
        return grad, coeff_grad, None, None


class MpartTorchInverse(torch.autograd.Function):
    """Inverse with a backward pass by the implicit-function rule (one
    InverseCoeffGrad call: dL/dc, dL/dr and dL/dx1 of the incoming gradient).
    The reference's TorchConditionalMapBase.inverse is not differentiable."""

    @staticmethod
    def forward(ctx, x1, r, coeffs, f):
        if coeffs is not None:
            c = coeffs.detach().to(device=r.device, dtype=torch.float64).contiguous()
            f.WrapCoeffs(c)
            ctx.c = c
        x1d = x1.detach().to(torch.float64)
        rd = r.detach().to(torch.float64)
        out = torch.zeros(f.outputDim, rd.shape[1], dtype=torch.float64, device=rd.device)
        f.InverseImpl(x1d, rd, out)
        ctx.f = f
        ctx.save_for_backward(x1, r, coeffs, out)
        return out.to(r.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        x1, r, coeffs, out = ctx.saved_tensors
        f = ctx.f
        if coeffs is not None:
            f.WrapCoeffs(ctx.c)
        extra = f.inputDim - f.outputDim
        n = out.shape[1]
        pts = torch.cat([x1.detach().to(torch.float64)[:extra].expand(extra, n), out], dim=0).contiguous()
        w = grad_out.detach().to(torch.float64).contiguous()
        want_c = coeffs is not None and coeffs.requires_grad
        cg = torch.zeros(f.numCoeffs, dtype=torch.float64, device=out.device) if want_c else None
        pg = torch.zeros(f.inputDim, n, dtype=torch.float64, device=out.device)
        f.InverseCoeffGradImpl(pts, w, cg, pg)
        g_x1 = None
        if x1.requires_grad:
            g_x1 = torch.zeros_like(x1, dtype=torch.float64)
            g_x1[:extra] = pg[:extra] if x1.shape[1] == n else pg[:extra].sum(dim=1, keepdim=True)
            g_x1 = g_x1.to(x1.dtype)
        g_r = pg[extra:].to(r.dtype) if r.requires_grad else None
        g_c = cg.to(coeffs.dtype) if want_c else None
        return g_x1, g_r, g_c, None


class TorchParameterizedFunctionBase(torch.nn.Module):
    """TorchParameterizedFunctionBase (bindings/python/package/torch.py):
    f(x) as a torch module, differentiable in x and in the coefficients (held
    as a Parameter when store_coeffs)."""

    def __init__(self, f, store_coeffs=True, dtype=torch.double, device="cuda"):
        super().__init__()
        self.f = f
        self.dtype = dtype
        if store_coeffs:
            self.coeffs = torch.nn.Parameter(torch.tensor(f.CoeffMap(), dtype=dtype, device=device))
        else:
            self.coeffs = None

    def forward(self, x, coeffs=None):
        coeffs = self.coeffs if coeffs is None else coeffs
        if coeffs is None:
            raise RuntimeError('Must either set store_coeffs=True in constructor or pass coeffs to forward function.')
        return MpartTorchAutograd.apply(x.T, coeffs, self.f, False).T


class TorchConditionalMapBase(torch.nn.Module):

    def __init__(self, f, store_coeffs=True, return_logdet=False, dtype=torch.double, device="cuda"):
        super().__init__()
        self.f = f
        self.return_logdet = return_logdet
        if store_coeffs:
            self.coeffs = torch.nn.Parameter(torch.tensor(f.CoeffMap(), dtype=dtype, device=device))
        else:
            self.coeffs = None

    def forward(self, x, coeffs=None):
        coeffs = self.coeffs if coeffs is None else coeffs
        if coeffs is None:
            raise RuntimeError('Must either set store_coeffs=True in constructor or pass coeffs to forward function.')
        if x.shape[1] != self.f.inputDim:
            raise ValueError(f'Input to map has wrong shape.  x has {x.shape[1]} columns but map expects input '
                             f'dimension of {self.f.inputDim}.')
        if self.return_logdet:
            y, logdet = MpartTorchAutograd.apply(x.T, coeffs, self.f, True)
            return y.T, logdet
        return MpartTorchAutograd.apply(x.T, coeffs, self.f, False).T

    def inverse(self, x, r, coeffs=None):
        """Inverse (bindings/python/package/torch.py inverse), differentiable in
        coeffs, r and the conditioning columns of x by the implicit-function rule."""
        coeffs = self.coeffs if coeffs is None else coeffs
        if x.shape[1] != self.f.inputDim and (x.shape[1] + r.shape[1]) == self.f.inputDim:
            x = torch.hstack([x, r])
        return MpartTorchInverse.apply(x.T, r.T, coeffs, self.f).T
