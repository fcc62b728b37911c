"""torch.autograd bridge for the replica energies (no counterpart in the
reference, which has no derivatives).

``replica_energy(positions, batch)`` returns the FP64 energy of every replica
of a ``ReplicaBatch`` (elastic + binding + field in the form whose
differences are the move dE) as a torch tensor that is differentiable with
respect to ``positions``, a [total_beads, 3] tensor with the replicas'
chains concatenated in order.  The forward uploads the positions and
rebuilds the densities; the backward scales ``cg_gradient``'s dE/dr by the
incoming gradient of each replica's energy.  Tangents and binding states are
the batch's current ones.  Derivatives with respect to the parameters are
``ReplicaBatch.gradient()``; through the Metropolis sampler they come from
reweighting (``ReplicaBatch.sensitivities``), not from autograd.
"""
import numpy as np
import torch


class ReplicaEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, batch):
        pos = positions.detach().to("cpu", torch.float64).numpy()
        chains, reps, off = [], [], 0
        for r, p in enumerate(batch.polymers):
            n = p.num_beads
            chains.append(dict(r=pos[off:off + n]))
            reps.append(np.full(n, r, dtype=np.int64))
            off += n
        if off != pos.shape[0]:
            raise ValueError("positions must hold every bead of every replica")
        batch.sim.set_chains(chains)
        batch.sim.deposit(-1)
        e = batch.sim.energies()[:, :3].sum(1)
        g, _ = batch.sim.gradient(positions=True, terms=False)
        ctx.save_for_backward(torch.from_numpy(g.astype(np.float64)), torch.from_numpy(np.concatenate(reps)))
        ctx.device = positions.device
        return torch.from_numpy(e).to(positions.device)

    @staticmethod
    def backward(ctx, grad_e):
        g, rep = ctx.saved_tensors
        scale = grad_e.detach().to("cpu", torch.float64)[rep]
        return (g * scale[:, None]).to(ctx.device), None


def replica_energy(positions: torch.Tensor, batch) -> torch.Tensor:
    """Energies [n_replicas] of ``batch`` at ``positions`` [total_beads, 3]."""
    return ReplicaEnergy.apply(positions, batch)
