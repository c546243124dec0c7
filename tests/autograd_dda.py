"""Test-only torch.autograd.Function over the C ABI: (Re chi, Im chi) per dipole -> (Cext, Cabs) of one incident
polarisation, with the backward pass given by adda_gb300_vjp_chi (one adjoint solve with the same matrix)."""
import numpy as np
import torch

import adda_gb300 as A


def cc_from_chi(s, chi, pol_index=0, relation="ldr"):
    """per-dipole polarisabilities and d(1/alpha)/dchi for susceptibilities chi [N] (m = sqrt(1 + 4 pi chi))"""
    m = np.sqrt(1 + 4 * np.pi * chi)
    cc = np.stack([A.polarizability(mi, s.kd, s.gridspace, s.prop, s.incpol[pol_index], relation) for mi in m])
    f = np.array([A.polarizability_dchi(mi, s.kd, s.gridspace, s.prop, s.incpol[pol_index], relation) for mi in m])
    return cc, f


class DdaCross(torch.autograd.Function):
    @staticmethod
    def forward(ctx_, chi_re, chi_im, ctx, s, pol_index, eps):
        chi = chi_re.detach().cpu().numpy() + 1j * chi_im.detach().cpu().numpy()
        cc, f = cc_from_chi(s, chi, pol_index)
        ctx.set_cc_dipole(0, cc)
        ctx.set_cc_dipole(1, cc)
        ctx.solve(s.einc[pol_index][None], prec="fp64", eps=eps)
        ce, ca = ctx.cross_sections(s.prop[None], s.incpol[pol_index][None])
        ge, ga = ctx.vjp_chi(0, s.prop, s.incpol[pol_index], f, eps=eps)
        ctx_.save_for_backward(torch.from_numpy(ge), torch.from_numpy(ga))
        return torch.tensor(ce[0], dtype=torch.float64), torch.tensor(ca[0], dtype=torch.float64)

    @staticmethod
    def backward(ctx_, g_ext, g_abs):
        ge, ga = ctx_.saved_tensors
        g = g_ext * ge + g_abs * ga
        return g[:, 0], g[:, 1], None, None, None, None
