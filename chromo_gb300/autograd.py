"""torch.autograd bridge for the replica energies (no counterpart in the
reference, which has no derivatives).

``replica_energy(positions, batch, tangents=None)`` returns the FP64 energy
of every replica of a ``ReplicaBatch`` (elastic + binding + field, in the
form whose differences are the per-move dE) as a CUDA tensor differentiable
with respect to ``positions`` and, when given, ``tangents`` -- [total_beads,
3] CUDA tensors with the replicas' chains concatenated in order.

Everything stays on the device: the forward copies the tensors into the
resident chains, rebuilds the densities, evaluates the energies and both
derivatives (dE/dr and dE/dt3 of the same energy, FP64) with device-pointer
entry points of the library, all on the current CUDA stream; the backward
scales them by the incoming gradient of each replica's energy.  t3 enters
only the elastic energy (chromo/polymers.pyx:1348-1381); t2 does not enter
the energy.  Binding states are the batch's current ones.  Derivatives with
respect to the parameters are ``ReplicaBatch.gradient()``; through the
Metropolis sampler they come from reweighting
(``ReplicaBatch.sensitivities``), not from autograd.
"""
import torch

from . import _native as nat


def _device_array(x, n, name):
    if not isinstance(x, torch.Tensor) or not x.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if tuple(x.shape) != (n, 3):
        raise ValueError(f"{name} must have shape [total_beads={n}, 3]")
    return x.detach().to(torch.float64).contiguous()


class ReplicaEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, tangents, batch):
        sim = batch.sim
        n = int(sim.n_beads.sum())
        pos = _device_array(positions, n, "positions")
        t3 = None if tangents is None else _device_array(tangents, n, "tangents")
        dev = pos.device
        stream = torch.cuda.current_stream(dev).cuda_stream
        L = nat.lib()
        nat.check(L.cg_set_chains_device(sim.h, pos.data_ptr(), None if t3 is None else t3.data_ptr(), stream))
        nat.check(L.cg_deposit_async(sim.h, stream))
        out = torch.empty((sim.R, 5), dtype=torch.float64, device=dev)
        nat.check(L.cg_energies_device(sim.h, out.data_ptr(), stream))
        want_t3 = tangents is not None and ctx.needs_input_grad[1]
        gr = torch.empty((n, 3), dtype=torch.float64, device=dev)
        gt = torch.empty((n, 3), dtype=torch.float64, device=dev) if want_t3 else None
        nat.check(L.cg_gradient_device(sim.h, gr.data_ptr(), None if gt is None else gt.data_ptr(), stream))
        counts = torch.as_tensor(sim.n_beads, dtype=torch.int64, device=dev)
        rep = torch.repeat_interleave(torch.arange(sim.R, device=dev), counts)
        ctx.want_t3 = want_t3
        ctx.save_for_backward(gr, gt if gt is not None else gr.new_empty(0), rep)
        return out[:, :3].sum(1)

    @staticmethod
    def backward(ctx, grad_e):
        gr, gt, rep = ctx.saved_tensors
        scale = grad_e.to(torch.float64)[rep][:, None]
        return gr * scale, (gt * scale if ctx.want_t3 else None), None


def replica_energy(positions: torch.Tensor, batch, tangents: torch.Tensor = None) -> torch.Tensor:
    """Energies [n_replicas] of ``batch`` at ``positions`` (and ``tangents``),
    [total_beads, 3] CUDA tensors."""
    return ReplicaEnergy.apply(positions, tangents, batch)
