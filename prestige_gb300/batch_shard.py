"""A batch of independent SPH systems shared out over ranks (one GPU each), no collective.

The batched step (pg_batch_create, one concatenated set of arrays with per-system constants)
runs every system on one GPU.  Over several ranks the systems are independent, so they are
bin-packed by particle count and every rank runs one batched handle of its own systems; nothing
is exchanged while the systems step.  The reference's pairwise loop runs over one set of slices
(prestige/src/codegen/simple_cpu.rs:7-19); each system here is one such set.

Packing (pack_systems): longest processing time first.  Systems in descending particle count
(ties by index) each go to the rank with the fewest particles so far (ties by rank), which keeps
the largest rank within 4/3 of the optimum (Graham 1969).  A rank keeps its systems in their
original order, so its batch is the original batch restricted to them.  Every rank computes the
same packing from the same counts.
"""
import heapq

import numpy as np

from .system import ParticleSystem

FIELDS = ("pos", "vel", "rho", "mass")


def pack_systems(counts, world):
    """Per rank, the ascending indices of the systems it runs (every system on exactly one rank)."""
    if world < 1:
        raise ValueError("world must be at least 1")
    counts = [int(c) for c in counts]
    if any(c < 0 for c in counts):
        raise ValueError("particle counts must be non-negative")
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for i in sorted(range(len(counts)), key=lambda i: (-counts[i], i)):
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + counts[i], r))
    return [sorted(s) for s in out]


def gpu_batch(configs, counts):
    return ParticleSystem.batch(configs, counts)


class ShardedBatch:
    """This rank's share of a batch of independent SPH systems.

    systems: list of {"config": make_config keyword dict, "n": particles, "fields": {"pos", "vel",
    "rho", "mass"}} (the format of prestige_gb300.workloads), the same list on every rank.
    make_batch(configs, counts) creates the batched handle (default: the GPU library)."""

    def __init__(self, systems, rank, world, make_batch=gpu_batch):
        if not 0 <= rank < world:
            raise ValueError("rank %d outside world %d" % (rank, world))
        self.rank = rank
        self.world = world
        self.n_systems = len(systems)
        self.counts = [int(w["n"]) for w in systems]
        self.packing = pack_systems(self.counts, world)
        self.mine = self.packing[rank]
        self.owner = [0] * self.n_systems
        for r, share in enumerate(self.packing):
            for i in share:
                self.owner[i] = r
        self.n = sum(self.counts[i] for i in self.mine)
        self.handle = None
        if self.mine:
            self.handle = make_batch([systems[i]["config"] for i in self.mine], [self.counts[i] for i in self.mine])
            try:
                for k in FIELDS:
                    self.handle.set(k, np.concatenate([np.asarray(systems[i]["fields"][k], np.float64)
                                                       for i in self.mine]))
            except BaseException:
                self.close()
                raise

    def particles_per_rank(self):
        return [sum(self.counts[i] for i in s) for s in self.packing]

    def enable_graph(self, enable=True):
        if self.handle is not None:
            self.handle.enable_graph(enable)

    def step(self, nsteps=1):
        if self.handle is not None:
            self.handle.step(nsteps)

    def step_async(self, nsteps=1):
        if self.handle is not None:
            self.handle.step_async(nsteps)

    def sync(self):
        if self.handle is not None:
            self.handle.sync()

    def fields(self, name):
        """{system index: this rank's array of the named field} for the rank's systems."""
        if self.handle is None:
            return {}
        a = np.asarray(self.handle.get(name))
        out, o = {}, 0
        for i in self.mine:
            out[i] = a[o:o + self.counts[i]].copy()
            o += self.counts[i]
        return out

    def gather(self, dist, names=("pos", "vel", "rho")):
        """Every system's named fields in the original system order, on every rank (host objects,
        after the run: not on the stepping path)."""
        mine = {name: self.fields(name) for name in names}
        parts = [None] * self.world
        dist.all_gather_object(parts, mine)
        out = []
        for i in range(self.n_systems):
            out.append(tuple(parts[self.owner[i]][name][i] for name in names))
        return out

    def close(self):
        if self.handle is not None:
            self.handle.close()
        self.handle = None
