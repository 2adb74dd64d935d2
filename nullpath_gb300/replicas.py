"""Multi-GPU replicas (one process per GPU, no data-path collective).

Every ray and every scene is independent, so N GPUs run N independent
replicas of a pass: rank r renders the workload with its own jitter seed,
and the job's time is the maximum over ranks.  The only collective is the
scalar max of the step time (NCCL on GPUs, gloo on CPU)."""
import torch


def rank_scene(scene, rank):
    """The rank's replica of `scene`: same camera and disk, jitter seeded with
    scene.seed + rank so that replicas trace different samples."""
    return scene.replace(seed=int(scene.seed) + int(rank))


def max_over_ranks(value, device=None):
    """Maximum of a Python float over the process group (the value itself
    without one)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rays_per_s(rays_per_rank, step_ms, world_size):
    """Whole-job throughput: all ranks' rays over the slowest rank's time."""
    return world_size * rays_per_rank / (step_ms * 1e-3)
