"""Whole-job figures of N independent replicas (one process per GPU).

The step does not shard across GPUs here: every rank runs its own replica of
the deck, with no data-path collective.  Only the timing is reduced: the
job's time is the slowest rank's, its work the sum over ranks.
"""


def reduce_replicas(seconds, particle_steps, dist=None, device="cpu"):
    """(job seconds = max over ranks, job particle-steps = sum over ranks,
    particle-steps/s) for this rank's figures; single-process when `dist` is
    None or not initialised."""
    if dist is None or not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(seconds), float(particle_steps), float(particle_steps) / float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    p = torch.tensor([float(particle_steps)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t.item()), float(p.item()), float(p.item()) / float(t.item())
