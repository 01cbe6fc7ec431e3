"""One SPH system split into slabs across ranks (one GPU each), with a halo exchange per step.

The reference runs its pairwise loop over one set of slices (prestige/src/codegen/simple_cpu.rs:
7-19); a system too large for one GPU is split here along one axis into slabs, one per rank, and
every rank runs the library's step on its own slab plus a halo, exchanging with its two
neighbours in between (torch.distributed point-to-point messages, host-staged).

Ownership.  The cut points along `axis` come from the initial positions (equal particle counts
per rank) and stay fixed; rank r owns the particles with cut[r] <= x_axis < cut[r+1] (the first
and last slabs are open).  Particles carry their global id.

One step (SlabSPH.step):
  1. Halo: each rank sends its lower neighbour the owned particles with x_axis < cut[r] + 2h,
     and its upper neighbour those with x_axis >= cut[r+1] - 2h (2h is the support: any
     neighbour of an owned particle of the other slab lies in that band).
  2. The local system is the owned and halo particles in global-id order, on the global cell
     grid.  Within a cell the neighbour walk therefore visits particles in the single-domain
     order, so the IEEE modes give the single-domain bits; fluid and wall particles keep their
     global roles (ids below the system's n_fluid are fluid).
  3. pg_step_stage(0): neighbour search and continuity pass.  The densities of the halo
     particles are incomplete there (part of their neighbourhood lies beyond the halo), so the
     owners send theirs (the same particles as in 1, in the same order) and they replace them.
  4. pg_step_stage(1): momentum pass with those densities; the owned particles keep the result.
  5. Migration: an owned particle whose new position lies in another slab moves to that rank (a
     step moves a particle by far less than a slab, so only to a neighbour).

The rank's handle is kept while its local particle and fluid counts stay the same (every field
is set anew each step) and is created again when they change.  No CPU fallback: `make_handle`
defaults to the GPU library.
"""
import numpy as np

from .system import ParticleSystem, make_config


def gpu_handle(cfg, n):
    return ParticleSystem(make_config(**cfg), n)


def _exchange(dist, peer, rows):
    """Send a float64 table to `peer` and receive the peer's table (same column count)."""
    import torch

    rows = np.ascontiguousarray(rows, np.float64)
    n_out = torch.tensor([rows.shape[0]], dtype=torch.int64)
    n_in = torch.zeros(1, dtype=torch.int64)
    req = dist.isend(n_out, peer)
    dist.recv(n_in, peer)
    req.wait()
    cols = rows.shape[1]
    incoming = torch.empty((int(n_in.item()), cols), dtype=torch.float64)
    reqs = [dist.isend(torch.from_numpy(rows), peer)] if rows.shape[0] else []
    if incoming.shape[0]:
        dist.recv(incoming, peer)
    for r in reqs:
        r.wait()
    return incoming.numpy()


class SlabSPH:
    """This rank's slab of one SPH system.

    cfg: make_config keyword dict of the whole system (n_fluid counted in global ids; < 0 or
    None: all fluid).  fields: the whole system's initial "pos", "vel", "rho", "mass" in global-id
    order (every rank passes the same arrays and keeps its own slab).  dist: an initialised
    torch.distributed module (any backend that moves CPU tensors point to point, e.g. gloo)."""

    def __init__(self, cfg, fields, dist, axis=0, make_handle=gpu_handle):
        self.cfg = dict(cfg)
        self.dist = dist
        self.rank = dist.get_rank()
        self.world = dist.get_world_size()
        self.axis = axis
        self.make_handle = make_handle
        pos = np.asarray(fields["pos"], np.float64)
        self.n_global, self.dim = pos.shape
        nf = self.cfg.get("n_fluid", -1)
        self.n_fluid_global = self.n_global if nf is None or nf < 0 else int(nf)
        self.halo = 2.0 * float(self.cfg["h"])
        q = np.quantile(pos[:, axis], [r / self.world for r in range(1, self.world)]) if self.world > 1 else []
        self.cuts = np.concatenate([[-np.inf], np.asarray(q, np.float64), [np.inf]])
        mine = self._owner(pos[:, axis]) == self.rank
        self.gid = np.nonzero(mine)[0].astype(np.int64)
        self.pos = pos[mine].copy()
        self.vel = np.asarray(fields["vel"], np.float64)[mine].copy()
        self.rho = np.asarray(fields["rho"], np.float64)[mine].copy()
        self.mass = np.asarray(fields["mass"], np.float64)[mine].copy()
        self._handle = None
        self._handle_key = None

    # -- helpers -----------------------------------------------------------------------------
    def _owner(self, x):
        return np.searchsorted(self.cuts, x, side="right") - 1

    def _rows(self, sel):
        return np.concatenate([self.gid[sel, None].astype(np.float64), self.pos[sel], self.vel[sel],
                               self.rho[sel, None], self.mass[sel, None]], axis=1)

    def _unpack(self, rows):
        d = self.dim
        return (rows[:, 0].astype(np.int64), rows[:, 1:1 + d], rows[:, 1 + d:1 + 2 * d], rows[:, 1 + 2 * d],
                rows[:, 2 + 2 * d])

    def _neighbours(self):
        """(peer rank, mask of owned particles to send it) for the lower and upper neighbour."""
        x = self.pos[:, self.axis]
        out = []
        if self.rank > 0:
            out.append((self.rank - 1, x < self.cuts[self.rank] + self.halo))
        if self.rank < self.world - 1:
            out.append((self.rank + 1, x >= self.cuts[self.rank + 1] - self.halo))
        return out

    # -- one step ----------------------------------------------------------------------------
    def step(self):
        d = self.dim
        peers = self._neighbours()
        # 1. halo
        halo = []
        for peer, sel in peers:
            halo.append(self._unpack(_exchange(self.dist, peer, self._rows(sel))))
        gid = np.concatenate([self.gid] + [h[0] for h in halo])
        pos = np.concatenate([self.pos] + [h[1] for h in halo])
        vel = np.concatenate([self.vel] + [h[2] for h in halo])
        rho = np.concatenate([self.rho] + [h[3] for h in halo])
        mass = np.concatenate([self.mass] + [h[4] for h in halo])
        # 2. the local system in global-id order
        order = np.argsort(gid, kind="stable")
        where = np.empty_like(order)
        where[order] = np.arange(order.size)  # local index of each concatenated row
        n_local = gid.size
        n_fluid = int(np.count_nonzero(gid < self.n_fluid_global))
        h = self._local_handle(n_local, n_fluid)
        try:
            h.set("pos", pos[order].reshape(n_local, d))
            h.set("vel", vel[order].reshape(n_local, d))
            h.set("rho", rho[order])
            h.set("mass", mass[order])
            # 3. continuity, then the owners' densities of the halo particles
            h.step_stage(0)
            rho_local = np.array(h.get("rho"), np.float64)
            own_local = where[:self.gid.size]
            start = self.gid.size
            for (peer, sel), hl in zip(peers, halo):
                back = _exchange(self.dist, peer, rho_local[own_local[sel]][:, None])
                rho_local[where[start:start + hl[0].size]] = back[:, 0]
                start += hl[0].size
            h.set("rho", rho_local)
            # 4. momentum; keep the owned particles
            h.step_stage(1)
            self.pos = np.asarray(h.get("pos"), np.float64).reshape(n_local, d)[own_local].copy()
            self.vel = np.asarray(h.get("vel"), np.float64).reshape(n_local, d)[own_local].copy()
            self.rho = np.asarray(h.get("rho"), np.float64)[own_local].copy()
        except BaseException:
            self.close()
            raise
        # 5. migration to the neighbour slabs
        dest = self._owner(self.pos[:, self.axis])
        if np.any(np.abs(dest - self.rank) > 1):
            raise RuntimeError("a particle moved further than one slab in one step")
        incoming = []
        for peer in (self.rank - 1, self.rank + 1):
            if 0 <= peer < self.world:
                incoming.append(self._unpack(_exchange(self.dist, peer, self._rows(dest == peer))))
        keep = dest == self.rank
        self.gid = np.concatenate([self.gid[keep]] + [m[0] for m in incoming])
        self.pos = np.concatenate([self.pos[keep]] + [m[1] for m in incoming])
        self.vel = np.concatenate([self.vel[keep]] + [m[2] for m in incoming])
        self.rho = np.concatenate([self.rho[keep]] + [m[3] for m in incoming])
        self.mass = np.concatenate([self.mass[keep]] + [m[4] for m in incoming])
        o = np.argsort(self.gid, kind="stable")
        self.gid, self.pos, self.vel, self.rho, self.mass = (self.gid[o], self.pos[o], self.vel[o], self.rho[o],
                                                             self.mass[o])

    def _local_handle(self, n_local, n_fluid):
        """The handle of the local system: the previous step's when the counts are the same (every
        field is set anew each step), else a new one."""
        if self._handle is not None and self._handle_key == (n_local, n_fluid):
            return self._handle
        self.close()
        self._handle = self.make_handle(dict(self.cfg, n_fluid=n_fluid), n_local)
        self._handle_key = (n_local, n_fluid)
        return self._handle

    def close(self):
        if self._handle is not None:
            self._handle.close()
        self._handle = None
        self._handle_key = None

    def run(self, nsteps):
        for _ in range(nsteps):
            self.step()

    def gather(self):
        """The whole system's pos, vel, rho in global-id order, on every rank."""
        parts = [None] * self.world
        self.dist.all_gather_object(parts, (self.gid, self.pos, self.vel, self.rho))
        gid = np.concatenate([p[0] for p in parts])
        o = np.argsort(gid)
        assert np.array_equal(gid[o], np.arange(self.n_global))
        return (np.concatenate([p[1] for p in parts])[o], np.concatenate([p[2] for p in parts])[o],
                np.concatenate([p[3] for p in parts])[o])
