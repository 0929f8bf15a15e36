"""torch.autograd view of the engine (for checking and for torch-side
optimisers): picks = EikonalPicks.apply(S, engine, shots, rx, rz).

S is the padded slowness (nxx, nzz) on the engine's device. Forward runs one
taped batched forward through the C ABI; backward runs the adjoint-state
reverse sweeps (sf_batch_adjoint) with the incoming pick gradients and
returns dJ/dS on the padded grid. Each forward supports one backward (the
tape is consumed), and only while the engine still holds that forward's tape:
a later forward, plan iteration or adjoint on the same engine replaces it,
and backward then raises instead of differentiating another batch.
"""
import torch


class EikonalPicks(torch.autograd.Function):
    @staticmethod
    def forward(ctx, S, engine, shots, rx, rz):
        if not S.is_cuda:
            raise ValueError("S must be a CUDA tensor on the engine's device")
        S = S.detach().contiguous()
        engine.set_slowness(S, padded=True)
        picks = torch.empty((len(shots), len(rx)), dtype=torch.float32, device=S.device)
        engine.batch_forward(shots, rx, rz, keep_tape=True, out=picks,
                             stream=torch.cuda.current_stream(S.device))
        engine.synchronize(torch.cuda.current_stream(S.device))
        ctx.engine = engine
        ctx.generation = engine.tape_generation
        ctx.shape = S.shape
        ctx.device = S.device
        return picks

    @staticmethod
    def backward(ctx, grad_picks):
        if ctx.engine.tape_generation != ctx.generation:
            raise RuntimeError("EikonalPicks.backward: the engine's tape belongs to a later call; run each "
                               "forward's backward before the next forward on the same engine, or use one "
                               "engine per forward")
        g = torch.empty(ctx.shape, dtype=torch.float32, device=ctx.device)
        stream = torch.cuda.current_stream(ctx.device)
        ctx.engine.batch_adjoint(grad_picks.detach().contiguous().float(), out=g, stream=stream)
        ctx.engine.synchronize(stream)
        return g, None, None, None, None
