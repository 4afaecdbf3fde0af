"""Differentiable CASCI energy: ``torch.autograd.Function`` over the GPU core.

Forward: CASCI ground-state energy of (h1, eri) (+ core energy) on the GPU
(the stored Hamiltonian, or the direct sigma when the stored matrix would not
fit on the device, as at CAS(14e,14o); Davidson; then the spin-resolved RDMs
of the converged vector).
Backward (Hellmann-Feynman, exact for the variational CI root):
    dE/dh1[p,q]      = gamma[p,q]       = (aa + bb)[p,q]
    dE/deri[p,q,r,s] = Gamma[p,q,r,s]   = (aaaa + bbbb + aabb + aabb^T)[p,q,r,s]
    dE/dcore         = 1
in the reference's RDM conventions (E = sum T.gamma + sum V.Gamma,
external/macis/tests/double_loop.cxx:197-241).  Integral tensors are
8-fold symmetric; a derivative along a symmetric perturbation is the sum of
the gradient over the perturbed orbit, which is what the finite-difference
checks compare.
"""
import numpy as np
import torch

from . import capi


def _rdm_pair(R):
    gamma = R["aa"] + R["bb"]
    Gamma = R["aaaa"] + R["bbbb"] + R["aabb"] + R["aabb"].transpose(2, 3, 0, 1)
    return gamma, Gamma


class CASCIEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h1, eri, core, nalpha, nbeta, tol, precision, device, max_m):
        T = h1.detach().double().cpu().numpy()
        V = eri.detach().double().cpu().numpy()
        n = T.shape[0]
        with capi.Context(device) as c:
            c.set_integrals(T, V)
            a, b = capi.fci_dets(n, nalpha, nbeta)
            c.set_dets(a, b)
            mixed = precision == "mixed"
            # stored matrix, or the direct sigma when it would not fit (CAS(14e,14o))
            c.build_operator(storage=capi.H_SPLIT32 if mixed else capi.H_FP64, max_m=max_m)
            E, C, info = c.davidson(tol=tol, max_m=max_m, precision=capi.PREC_MIXED if mixed else capi.PREC_FP64)
            R = c.rdms_spin_dep(C)
        gamma, Gamma = _rdm_pair(R)
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(gamma)).to(h1.device),
                              torch.from_numpy(np.ascontiguousarray(Gamma)).to(eri.device))
        ctx.core_device = core.device
        return torch.tensor(E, dtype=torch.float64, device=h1.device) + core.double()

    @staticmethod
    def backward(ctx, gE):
        gamma, Gamma = ctx.saved_tensors
        g = gE.double()
        return (g * gamma, g * Gamma, g.to(ctx.core_device), None, None, None, None, None, None)


def casci_energy(h1, eri, nalpha, nbeta, core=None, tol=1e-10, precision="fp64", device=0, max_m=200):
    """E(h1, eri) = CASCI ground-state energy, differentiable w.r.t. h1, eri, core."""
    if core is None:
        core = torch.zeros((), dtype=torch.float64, device=h1.device)
    return CASCIEnergy.apply(h1, eri, core, int(nalpha), int(nbeta), float(tol), precision, int(device), int(max_m))


def rdms_as_gradients(h1, eri, nalpha, nbeta, tol=1e-10, precision="fp64"):
    """(E, dE/dh1, dE/deri) through autograd (convenience for callers)."""
    h1 = h1.detach().clone().requires_grad_(True)
    eri = eri.detach().clone().requires_grad_(True)
    E = casci_energy(h1, eri, nalpha, nbeta, tol=tol, precision=precision)
    E.backward()
    return E.detach(), h1.grad, eri.grad
