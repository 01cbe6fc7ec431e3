"""One SPH or DEM system split into slabs across ranks (one GPU each), with a halo exchange per step.

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

SlabDEM (below) is the same decomposition for a DEM system: a band of 2 r_max, one stage per
step, and the tangential contact history carried in global ids.
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


# ------------------------------------------------------------------------------------------------
# DEM slabs
# ------------------------------------------------------------------------------------------------
WALL_ID = 0xFFFFFFF0  # partner codes WALL_ID + face in the contact history
NO_PARTNER = 0xFFFFFFFF  # an empty history slot (the slots after a particle's last contact)


class SlabDEM:
    """This rank's slab of one DEM system (pg_step: the contact pass with its integrator).

    The same cuts, ownership and migration as SlabSPH, along `axis` (the longest, z, by default).
    One step is one stage: a sphere's force and torque depend on the positions, velocities and
    spins of the spheres in contact with it and on its own tangential history, so
      1. each rank sends each neighbour its owned spheres within 2 r_max of the shared cut (any
         contact partner of an owned sphere, at a distance below r_i + r_j <= 2 r_max, is owned or
         in that band on the other side);
      2. the local system is the owned and halo spheres in global-id order on the global cell
         grid and walls, so the contact walk meets the spheres of a cell in the single-domain order;
      3. the owned spheres' tangential history (partner global ids, walls as WALL_ID + face) is
         translated to local ids and set; halo spheres start empty (their results are dropped);
         a partner absent from the local system cannot be in contact, so its entry is dropped (the
         history holds the contacts of the last step, in the order found);
      4. one step; the owned spheres keep the result and their history, translated back to
         global ids;
      5. spheres that crossed a cut migrate, with their history.

    fields: the whole system's "pos", "vel", "omega", "radius", "mass" in global-id order, plus
    optionally "history": (partner ids (n, C), springs (n, C, 3)) in global ids."""

    def __init__(self, cfg, fields, dist, axis=2, make_handle=gpu_handle):
        self.cfg = dict(cfg)
        self.dist = dist
        self.rank = dist.get_rank()
        self.world = dist.get_world_size()
        self.axis = axis
        self.make_handle = make_handle
        pos = np.asarray(fields["pos"], np.float64)
        self.n_global = pos.shape[0]
        self.C = int(self.cfg.get("contact_capacity", 16))
        self.halo = 2.0 * float(self.cfg["r_max"])
        q = np.quantile(pos[:, axis], [r / self.world for r in range(1, self.world)]) if self.world > 1 else []
        self.cuts = np.concatenate([[-np.inf], np.asarray(q, np.float64), [np.inf]])
        mine = self._owner(pos[:, axis]) == self.rank
        self.gid = np.nonzero(mine)[0].astype(np.int64)
        self.f = {k: np.asarray(fields[k], np.float64)[mine].copy() for k in ("pos", "vel", "omega", "radius", "mass")}
        if "history" in fields:
            hp, hx = fields["history"]
            self.hpid = np.asarray(hp, np.uint32).reshape(self.n_global, self.C)[mine].copy()
            self.hxi = np.asarray(hx, np.float64).reshape(self.n_global, self.C, 3)[mine].copy()
        else:
            self.hpid = np.full((self.gid.size, self.C), NO_PARTNER, np.uint32)
            self.hxi = np.zeros((self.gid.size, self.C, 3))
        self._handle = None
        self._handle_n = None

    def _owner(self, x):
        return np.searchsorted(self.cuts, x, side="right") - 1

    def _neighbours(self):
        x = self.f["pos"][:, self.axis]
        out = []
        if self.rank > 0:
            out.append((self.rank - 1, x < self.cuts[self.rank] + self.halo))
        if self.rank < self.world - 1:
            out.append((self.rank + 1, x >= self.cuts[self.rank + 1] - self.halo))
        return out

    # rows: gid, pos (3), vel (3), omega (3), radius, mass [, partner ids (C), springs (3C)]
    def _rows(self, sel, history):
        cols = [self.gid[sel, None].astype(np.float64), self.f["pos"][sel], self.f["vel"][sel], self.f["omega"][sel],
                self.f["radius"][sel, None], self.f["mass"][sel, None]]
        if history:
            cols += [self.hpid[sel].astype(np.float64), self.hxi[sel].reshape(-1, 3 * self.C)]
        return np.concatenate(cols, axis=1)

    def _unpack(self, rows, history):
        out = {"gid": rows[:, 0].astype(np.int64), "pos": rows[:, 1:4], "vel": rows[:, 4:7], "omega": rows[:, 7:10],
               "radius": rows[:, 10], "mass": rows[:, 11]}
        if history:
            C = self.C
            out["hpid"] = rows[:, 12:12 + C].astype(np.uint32)
            out["hxi"] = rows[:, 12 + C:12 + 4 * C].reshape(-1, C, 3)
        return out

    @staticmethod
    def _compact(hp, hx, keep):
        """Keep the marked entries of each row in order, the rest of the row empty."""
        out_p = np.full_like(hp, NO_PARTNER)
        out_x = np.zeros_like(hx)
        r, c = np.nonzero(keep)
        dst = (np.cumsum(keep, axis=1) - 1)[r, c]
        out_p[r, dst] = hp[r, c]
        out_x[r, dst] = hx[r, c]
        return out_p, out_x

    def _history_to_local(self, g2l):
        hp = self.hpid.astype(np.int64)
        live = np.cumprod(hp != NO_PARTNER, axis=1).astype(bool)  # up to the first empty slot
        particle = live & (hp < WALL_ID)
        mapped = np.where(particle, g2l[np.where(particle, hp, 0)], hp)
        keep = live & ((hp >= WALL_ID) | (mapped >= 0))
        return self._compact(mapped.astype(np.uint32), self.hxi, keep)

    @staticmethod
    def _history_to_global(hp, gid_local):
        hp = np.asarray(hp, np.int64)
        particle = hp < WALL_ID
        return np.where(particle, gid_local[np.where(particle, hp, 0)], hp).astype(np.uint32)

    def step(self):
        peers = self._neighbours()
        halo = [self._unpack(_exchange(self.dist, peer, self._rows(sel, False)), False) for peer, sel in peers]
        gid = np.concatenate([self.gid] + [h["gid"] for h in halo])
        order = np.argsort(gid, kind="stable")
        where = np.empty_like(order)
        where[order] = np.arange(order.size)
        n_local = gid.size
        gid_local = gid[order]
        g2l = np.full(self.n_global, -1, np.int64)
        g2l[gid_local] = np.arange(n_local)
        own_local = where[:self.gid.size]
        h = self._local_handle(n_local)
        try:
            for k in ("pos", "vel", "omega", "radius", "mass"):
                h.set(k, np.concatenate([self.f[k]] + [x[k] for x in halo])[order])
            hp_own, hx_own = self._history_to_local(g2l)
            hp = np.full((n_local, self.C), NO_PARTNER, np.uint32)
            hx = np.zeros((n_local, self.C, 3))
            hp[own_local] = hp_own
            hx[own_local] = hx_own
            h.set_dem_history(hp, hx)
            h.step(1)
            for k in ("pos", "vel", "omega"):
                self.f[k] = np.asarray(h.get(k), np.float64).reshape(n_local, 3)[own_local].copy()
            hp, hx = h.dem_history()
            self.hpid = self._history_to_global(np.asarray(hp).reshape(n_local, self.C)[own_local], gid_local)
            self.hxi = np.asarray(hx, np.float64).reshape(n_local, self.C, 3)[own_local].copy()
        except BaseException:
            self.close()
            raise
        # migration to the neighbour slabs, with the history
        dest = self._owner(self.f["pos"][:, self.axis])
        if np.any(np.abs(dest - self.rank) > 1):
            raise RuntimeError("a sphere moved further than one slab in one step")
        incoming = []
        for peer in (self.rank - 1, self.rank + 1):
            if 0 <= peer < self.world:
                incoming.append(self._unpack(_exchange(self.dist, peer, self._rows(dest == peer, True)), True))
        keep = dest == self.rank
        self.gid = np.concatenate([self.gid[keep]] + [m["gid"] for m in incoming])
        for k in self.f:
            self.f[k] = np.concatenate([self.f[k][keep]] + [m[k] for m in incoming])
        self.hpid = np.concatenate([self.hpid[keep]] + [m["hpid"] for m in incoming])
        self.hxi = np.concatenate([self.hxi[keep]] + [m["hxi"] for m in incoming])
        o = np.argsort(self.gid, kind="stable")
        self.gid = self.gid[o]
        for k in self.f:
            self.f[k] = self.f[k][o]
        self.hpid, self.hxi = self.hpid[o], self.hxi[o]

    def _local_handle(self, n_local):
        if self._handle is not None and self._handle_n == n_local:
            return self._handle
        self.close()
        self._handle = self.make_handle(dict(self.cfg), n_local)
        self._handle_n = n_local
        return self._handle

    def close(self):
        if self._handle is not None:
            self._handle.close()
        self._handle = None
        self._handle_n = None

    def run(self, nsteps):
        for _ in range(nsteps):
            self.step()

    def gather(self):
        """The whole system's pos, vel, omega and history (global ids) in global-id order, on every
        rank."""
        parts = [None] * self.world
        self.dist.all_gather_object(parts, (self.gid, self.f["pos"], self.f["vel"], self.f["omega"], self.hpid,
                                            self.hxi))
        gid = np.concatenate([p[0] for p in parts])
        o = np.argsort(gid)
        assert np.array_equal(gid[o], np.arange(self.n_global))
        return tuple(np.concatenate([p[i] for p in parts])[o] for i in range(1, 6))
