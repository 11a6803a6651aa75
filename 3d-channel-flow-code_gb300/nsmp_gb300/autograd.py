"""torch.autograd.Function around the library's discrete adjoint.

`wall_shear_objective(solver, fx, state, nsteps, ckpt_every)` returns the
time-averaged wall shear stress J of `nsteps` SSP-RK3 steps run from `state`
with the per-cell body force `fx` ((N0, NZ) tensor, ghost layers ignored) as a
0-d tensor.  Its backward pass is the gradient dJ/dfx computed by
nsmp_adjoint in the same call, so `J.backward()` fills `fx.grad`.

The solver runs on its own CUDA stream and host arrays cross the C-ABI;
torch is only the harness here.
"""
import numpy as np
import torch


def capture_state(solver):
    """The state nsmp_upload_state takes: (cell fields u, v, w, p), (5 face
    fluxes), (3 AB2 histories)."""
    import nsmp_gb300 as ng
    cells = [solver.download(f) for f in (ng.F_U, ng.F_V, ng.F_W, ng.F_P)]
    faces = [solver.download(f) for f in (ng.F_U1FACE, ng.F_U2FACE, ng.F_U3FACE, ng.F_UTFACE, ng.F_UBFACE)]
    hist = [solver.download(f) for f in (ng.F_RHSU, ng.F_RHSV, ng.F_RHSW)]
    return cells, faces, hist


class WallShearObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, fx, solver, state, nsteps, ckpt_every):
        cells, faces, hist = state
        solver.upload_state(*cells, faces, hist, 0)
        f = np.asfortranarray(fx.detach().to("cpu", torch.float64).numpy())
        J, grad, rc = solver.adjoint(int(nsteps), int(ckpt_every), f)
        g = torch.from_numpy(np.ascontiguousarray(grad)).to(device=fx.device, dtype=fx.dtype)
        ctx.save_for_backward(g)
        ctx.status = rc
        return fx.new_tensor(J)

    @staticmethod
    def backward(ctx, gJ):
        (g,) = ctx.saved_tensors
        return gJ * g, None, None, None, None


def wall_shear_objective(solver, fx, state, nsteps, ckpt_every):
    return WallShearObjective.apply(fx, solver, state, nsteps, ckpt_every)
