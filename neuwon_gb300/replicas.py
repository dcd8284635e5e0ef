"""Several GPUs as replicas: the path shards by neuron with no exchange (the
propagator is block-diagonal by neuron and mechanisms are per instance), so
each rank advances its own batch and nothing crosses ranks in the data path.
The whole-job throughput is the segments of all ranks times the steps over
the slowest rank's time (a barrier brackets the timed region)."""
import numpy as np


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


# ------------------------------------------------------- partitioned networks
# A network whose neurons are split across ranks has one real exchange step:
# spikes.  Every rank keeps the spike ring of all neurons (bit t mod R of neuron
# j = AP at step t) but writes only its own neurons' words; a synapse reads the
# ring at step - delay.  After an epoch of at most the shortest delay, the ranks
# sum their rings with the other ranks' neurons zeroed, so every rank holds
# every neuron's bits before any synapse can need them.

def own_part(ring, offset, count):
    """The ring with every neuron outside [offset, offset + count) zeroed."""
    out = np.zeros_like(ring)
    out[offset:offset + count] = ring[offset:offset + count]
    return out


def exchange_rings(ring, offset, count, dist=None):
    """Sum of all ranks' own parts (what every rank installs after an epoch)."""
    part = own_part(ring, offset, count)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return part
    import torch
    t = torch.from_numpy(part.astype(np.int64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.numpy().astype(ring.dtype)


class SpikeExchange:
    """Drives one rank's model of a partitioned network: advance an epoch, then
    exchange spike rings.  ``reduce`` sums the ranks' own parts (default: the
    torch.distributed process group; a plain function for emulated ranks)."""

    def __init__(self, model, dist=None, reduce=None):
        self.model = model
        self.dist = dist
        self.reduce = reduce

    def ring(self):
        ctx = self.model._ctx
        N = ctx.get_option("spike_neurons")
        W = ctx.get_option("synapse_ring_words")
        return ctx.get_data("Synapse.spike_ring", N * W, np.uint32).reshape(N, W)

    def own(self):
        m = self.model
        return own_part(self.ring(), m._ctx.get_option("spike_neuron_offset"), len(m._neuron_root))

    def install(self, total):
        self.model._ctx.set_data("Synapse.spike_ring", np.ascontiguousarray(total.ravel()))

    def exchange(self):
        if self.reduce is not None:
            self.install(self.reduce(self))
            return
        m = self.model
        self.install(exchange_rings(self.ring(), m._ctx.get_option("spike_neuron_offset"), len(m._neuron_root),
                                    self.dist))


