"""Force-matching fits over the GPU adjoint (mdgpu_fm_loss_grad,
mdgpu_energy_grad) as torch.autograd.Functions.

The functions take the raw parameters of the force path as float64 CPU
tensors -- the potential table ``potpar`` [max_id*max_id, 8], the per-site
charges ``chg`` [nsites] and ``alpha`` [] -- so that any parametrisation
(for water: epsilon, sigma, q_H with q_M = -2 q_H) is ordinary torch code in
front of them and autograd chains through it.  Their forward pass evaluates
the loss (or energy) with the GPU force path; their backward pass calls the
adjoint, which re-runs the forward evaluation and walks the link cells again
(no pair list is kept between the passes).

PyTorch is host plumbing here: the arithmetic is the library's CUDA kernels.
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional, Sequence

import numpy as np
import torch

from .forcefield import ForceField
from .system import CONV_E, CONV_Q, System


@dataclasses.dataclass
class FitProblem:
    """Frames (site co-ordinates [3, N] and fractional centres of mass) with
    their reference forces, evaluated by one ForceField.  The loss is
    weight * sum over frames and sites of |F - F_ref|^2."""
    ff: ForceField
    frames: Sequence[np.ndarray]
    cofms: Sequence[np.ndarray]
    f_refs: Optional[Sequence[np.ndarray]] = None
    weight: float = 1.0

    def _set(self, potpar, chg, alpha):
        self.ff.set_params(potpar.detach().cpu().numpy(), chg.detach().cpu().numpy(), float(alpha))


def _as_grads(gp, gq, ga, like):
    return (torch.from_numpy(gp.reshape(like[0].shape)).to(like[0]), torch.from_numpy(gq).to(like[1]),
            torch.tensor(ga, dtype=like[2].dtype))


class ForceMatchLoss(torch.autograd.Function):
    """loss = ForceMatchLoss.apply(potpar, chg, alpha, problem)"""

    @staticmethod
    def forward(ctx, potpar, chg, alpha, problem: FitProblem):
        problem._set(potpar, chg, alpha)
        total = 0.0
        for site, cm, fr in zip(problem.frames, problem.cofms, problem.f_refs):
            f, _, _ = problem.ff.forces(site, cm)
            total += problem.weight * float(np.sum((f - fr) ** 2))
        ctx.problem = problem
        ctx.save_for_backward(potpar, chg, alpha)
        return torch.tensor(total, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        potpar, chg, alpha = ctx.saved_tensors
        pb: FitProblem = ctx.problem
        pb._set(potpar, chg, alpha)
        gp = gq = None
        ga = 0.0
        for site, cm, fr in zip(pb.frames, pb.cofms, pb.f_refs):
            _, g = pb.ff.fm_loss_grad(fr, pb.weight, site, cm)
            gp = g["potpar"] if gp is None else gp + g["potpar"]
            gq = g["chg"] if gq is None else gq + g["chg"]
            ga += g["alpha"]
        gp_t, gq_t, ga_t = _as_grads(gp, gq, ga, (potpar, chg, alpha))
        return grad_out * gp_t, grad_out * gq_t, grad_out * ga_t, None


class EnergySum(torch.autograd.Function):
    """energy = EnergySum.apply(potpar, chg, alpha, problem): the sum of the
    potential energies of the problem's frames."""

    @staticmethod
    def forward(ctx, potpar, chg, alpha, problem: FitProblem):
        problem._set(potpar, chg, alpha)
        total = 0.0
        for site, cm in zip(problem.frames, problem.cofms):
            _, pe, _ = problem.ff.forces(site, cm)
            total += float(pe[0] + pe[1])
        ctx.problem = problem
        ctx.save_for_backward(potpar, chg, alpha)
        return torch.tensor(total, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        potpar, chg, alpha = ctx.saved_tensors
        pb: FitProblem = ctx.problem
        pb._set(potpar, chg, alpha)
        gp = gq = None
        ga = 0.0
        for site, cm in zip(pb.frames, pb.cofms):
            _, g = pb.ff.energy_grad(site, cm)
            gp = g["potpar"] if gp is None else gp + g["potpar"]
            gq = g["chg"] if gq is None else gq + g["chg"]
            ga += g["alpha"]
        gp_t, gq_t, ga_t = _as_grads(gp, gq, ga, (potpar, chg, alpha))
        return grad_out * gp_t, grad_out * gq_t, grad_out * ga_t, None


# ---------------------------------------------------------------------------
# rigid 4-site water (moldy_gb300.system.water): O id 1, H id 2, M id 3
# ---------------------------------------------------------------------------
def water_tables(eps: torch.Tensor, sigma: torch.Tensor, q_h: torch.Tensor, base: System):
    """(potpar [max_id^2, 8], chg [N]) of the water model for LJ epsilon
    (kJ/mol), sigma (Å) and the H charge (e), with q_M = -2 q_H keeping each
    molecule neutral; every other table entry is taken from ``base``."""
    M = base.max_id
    pot = torch.as_tensor(np.asarray(base.potpar, np.float64).reshape(M, M, 8)).clone()
    idx = (torch.tensor([1, 1]), torch.tensor([1, 1]), torch.tensor([0, 1]))
    pot = pot.index_put(idx, torch.stack([4.0 * eps / CONV_E, sigma]))
    qid = torch.stack([torch.zeros((), dtype=torch.float64), torch.zeros((), dtype=torch.float64),
                       q_h, -2.0 * q_h]) / CONV_Q
    chg = qid[torch.as_tensor(base.site_ids(), dtype=torch.long)]
    return pot.reshape(M * M, 8), chg


def water_frames(base: System, nframes: int, seed: int, displacement: float = 0.1) -> List[System]:
    """Seeded frames of a water system: every molecule's centre of mass
    displaced by a Gaussian of ``displacement`` Å rms and rotated to a fresh
    uniform-random orientation, sites wrapped into the cell."""
    from .system import _random_quaternions, _rotation_matrices, _wrap_sites
    rng = np.random.default_rng(seed)
    sp = base.species[0]
    h = np.asarray(base.h, np.float64)
    out = []
    for _ in range(nframes):
        dc = rng.normal(0.0, displacement, (sp.nmols, 3)) @ np.linalg.inv(h).T
        cf = base.c_of_m + dc
        cf -= np.floor(cf + 0.5)
        R = _rotation_matrices(_random_quaternions(rng, sp.nmols))
        com = cf @ h.T
        x = (com[:, None, :] + np.einsum("mij,sj->msi", R, sp.p_f_sites)).reshape(-1, 3).T
        out.append(base.with_sites(_wrap_sites(h, x.copy()), cf))
    return out
