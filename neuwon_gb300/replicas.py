"""Several GPUs as replicas: the path shards by neuron with no exchange (the
propagator is block-diagonal by neuron and mechanisms are per instance), so
each rank advances its own batch and nothing crosses ranks in the data path.
The whole-job throughput is the segments of all ranks times the steps over
the slowest rank's time (a barrier brackets the timed region)."""


def replica_seed(rank):
    """Seed of a rank's batch: rank r generates the trees with seeds r*N + k + 1."""
    return int(rank)


def aggregate(local_ms, local_segments, steps, dist=None, device="cpu"):
    """(max ms over ranks, total segments, whole-job segment-steps/s)."""
    ms, segments = float(local_ms), int(local_segments)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        s = torch.tensor([segments], dtype=torch.int64, device=device)
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
        ms, segments = float(t.item()), int(s.item())
    return {"ms": ms, "segments": segments, "value": segments * steps / (ms * 1e-3)}
