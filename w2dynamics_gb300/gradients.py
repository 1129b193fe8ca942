"""Derivatives of configuration weights (the backward pass).

For a fixed configuration the weight is w = det H(Delta) * Tr[...](H_loc).
`cthyb_batch_gradients` (device kernel `k_grad`) returns per chain
d log|det| / d Delta on the F(tau) grid and d log|trace| along parameter
directions of H_loc given as per-eigenstate energy derivatives.  Here:

* `density_density_directions`: the energy derivatives of the
  density-density local Hamiltonian with respect to the one-particle levels
  eps_f (the diagonal of `muimp`, solver sign) and the interaction
  parameters (U, J) with U' = U - 2J (the parametrisation of
  `interaction.Density`, w2dyn/dmft/interaction.py:171-213), per eigenstate
  of a monomial model (eigenstates are Fock states);
* `LogWeight`: a torch.autograd.Function whose forward returns log|w| of
  every chain's current configuration and whose backward applies the chain
  rule with the kernel's gradients;
* `score_covariance`: d<O>/dtheta = <O g> - <O><g> from per-measurement
  samples of an observable O and g = d log|w| / dtheta (score-function
  estimator; the G(tau) estimator itself does not depend on H_loc).
"""
import numpy as np

from . import problems as P


def _occupations(nd, fock):
    fock = np.asarray(fock, np.int64)
    nf = 2 * nd
    n = np.zeros((nf, len(fock)))
    for f in range(nf):
        n[f] = (fock >> (f // 2 + nd * (f % 2))) & 1
    return n


def interaction_energy(nd, umatrix, fock):
    """<n|1/2 sum U_ijkl c+_i c+_j c_l c_k|n> = 1/2 sum_{i!=j} (U_ijij - U_ijji) n_i n_j
    for Fock states (flavour f = 2b + s)."""
    u = np.asarray(umatrix, np.float64).reshape((2 * nd,) * 4)
    n = _occupations(nd, fock)
    e = np.zeros(n.shape[1])
    for i in range(2 * nd):
        for j in range(2 * nd):
            if i != j:
                e += 0.5 * (u[i, j, i, j] - u[i, j, j, i]) * n[i] * n[j]
    return e


def density_density_directions(nd, fock_states):
    """dE (2Nd + 2, nstates): rows d/d eps_f (f = 2b + s), d/dU, d/dJ for
    E = sum_f eps_f n_f + E_int(U, U - 2J, J) at the eigenstates whose Fock
    states are `fock_states` (a monomial model's `fock_states`)."""
    n = _occupations(nd, fock_states)
    du = interaction_energy(nd, P.flat_umatrix(P.umatrix_density(nd, 1.0, 1.0, 0.0)), fock_states)
    dj = interaction_energy(nd, P.flat_umatrix(P.umatrix_density(nd, 0.0, -2.0, 1.0)), fock_states)
    return np.vstack([n, du[None, :], dj[None, :]])


def _torch():
    import torch
    return torch


class _LogWeightFn:
    """Built lazily so that importing this module does not need torch."""
    cls = None


def LogWeight():
    """torch.autograd.Function: log_w = LogWeight().apply(ftau, theta, batch, dE)
    with ftau the (Nd, 2, Nftau) grid and theta the parameters the batch was
    built with (their values are the batch's; they carry the gradient), dE
    the (nparams, nstates) energy derivatives of the parameter directions
    (numpy or torch, or None).  Everything runs on the device: the forward
    value comes from the weights the chains carry
    (cthyb_batch_log_weights_device, no kernel walk); the backward launches
    the gradient kernel into device tensors (cthyb_batch_gradients_device)
    only when a gradient is requested and contracts with grad_out on the
    device.  Gradients are returned on the devices of ftau and theta."""
    if _LogWeightFn.cls is not None:
        return _LogWeightFn.cls
    torch = _torch()

    class Fn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, ftau, theta, batch, dE):
            dev = torch.device("cuda")
            lw = torch.empty((batch.nchains, 2), dtype=torch.float64, device=dev)
            batch.log_weights_device(lw, stream=torch.cuda.current_stream().cuda_stream)
            ctx.batch = batch
            ctx.dE = None if dE is None else torch.as_tensor(dE, dtype=torch.float64).to(dev)
            ctx.fshape, ctx.fdev, ctx.tdev = ftau.shape, ftau.device, theta.device
            return lw.sum(dim=1).to(ftau.device, ftau.dtype)

        @staticmethod
        def backward(ctx, grad_out):
            b, dE = ctx.batch, ctx.dE
            dev = torch.device("cuda")
            n = b.nchains
            nf, nft = 2 * ctx.fshape[0], ctx.fshape[2]
            npar = 0 if dE is None else int(dE.shape[0])
            gd = torch.empty((n, nf, nft), dtype=torch.float64, device=dev)
            gp = torch.empty((n, max(npar, 1)), dtype=torch.float64, device=dev)
            lw = torch.empty((n, 2), dtype=torch.float64, device=dev)
            b.gradients_device(dE, gd, gp if npar else None, lw, stream=torch.cuda.current_stream().cuda_stream)
            go = grad_out.to(dev, torch.float64)
            g_f = torch.einsum("c,cfj->fj", go, gd).reshape(ctx.fshape)
            g_t = go @ gp[:, :npar] if npar else torch.zeros(0, dtype=torch.float64, device=dev)
            return g_f.to(ctx.fdev), g_t.to(ctx.tdev), None, None

    _LogWeightFn.cls = Fn
    return Fn


def score_covariance(obs, scores):
    """d<O>/dtheta from samples: obs (nsamples, ...) and scores (nsamples,
    nparams) -> (nparams, ...) = <O g> - <O><g>."""
    obs = np.asarray(obs, np.float64)
    g = np.asarray(scores, np.float64)
    o = obs.reshape(len(obs), -1)
    cov = (g.T @ o) / len(obs) - np.outer(g.mean(axis=0), o.mean(axis=0))
    return cov.reshape((g.shape[1],) + obs.shape[1:])
