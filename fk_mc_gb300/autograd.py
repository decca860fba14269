"""torch.autograd.Function wrappers of the free-energy derivatives.

`FreeEnergy.apply(U, t, mu, beta, solver, lattice_ids, f)` returns
F = -logZ/beta for every configuration (tensor of shape (B,)); its backward
returns dF/dU, dF/dt, dF/dmu, dF/dbeta. Both come from one call of the C ABI
entry point fkg_free_energy_grad: the eigendecomposition that F needs is the
one the backward kernels (dF/dH = V diag(fermi) V^T and its reductions) use,
so the forward pass computes the derivatives once and the backward pass only
scales them by the incoming gradient. When no input needs a gradient (no
backward can follow), the forward pass is the plain eigen-solve + logZ
(fkg_eigh_logz) and no derivative kernel runs.

The full dF/dH (the density matrix rho) is available from
`Solver.free_energy_grad(..., rho=True)`.
"""
import numpy as np
import torch


def _np(x, B):
    return np.broadcast_to(x.detach().cpu().double().numpy() if torch.is_tensor(x) else np.asarray(x, float), (B,))


class FreeEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U, t, mu, beta, solver, lattice_ids, f):
        ids = np.asarray(lattice_ids, dtype=np.int32)
        B = ids.size
        dev = U.device if torch.is_tensor(U) else torch.device("cpu")
        ctx.shapes = [tuple(x.shape) if torch.is_tensor(x) else () for x in (U, t, mu, beta)]
        if not any(ctx.needs_input_grad[:4]):
            Ub, mub, bb = _np(U, B), _np(mu, B), _np(beta, B)
            ns = [solver.sizes[int(i)] for i in ids]
            fa = np.asarray(f, dtype=np.float64).ravel()
            cut = np.cumsum([0] + ns)
            diag = np.concatenate([-mub[c] + Ub[c] * fa[cut[c]:cut[c + 1]] for c in range(B)])
            out = solver.eigh_logz(ids, diag, bb)
            return torch.as_tensor(-out["logz"] / bb, dtype=torch.float64, device=dev)
        out = solver.free_energy_grad(ids, f, _np(U, B), _np(mu, B), _np(t, B), _np(beta, B))
        grads = [torch.as_tensor(out[k], dtype=torch.float64, device=dev) for k in ("dU", "dt", "dmu", "dbeta")]
        ctx.save_for_backward(*grads)
        return torch.as_tensor(out["F"], dtype=torch.float64, device=dev)

    @staticmethod
    def backward(ctx, gF):
        gs = []
        for g, shape in zip(ctx.saved_tensors, ctx.shapes):
            v = gF * g
            gs.append(v.sum() if shape == () else v.reshape(shape) if v.numel() == int(np.prod(shape)) else v.sum())
        return gs[0], gs[1], gs[2], gs[3], None, None, None
