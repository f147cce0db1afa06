"""Forward/backward pair of the topology-frozen adjoint, and terrain fitting.

No counterpart in the reference (it has no derivatives).  :class:`Adjoint`
keeps the device buffers of one chunk batch and drives ``uww_forward`` /
``uww_backward`` / ``uww_height_loss`` of libuww_gb300.so; :class:`TerrainFit`
is the Adam loop that fits theta = (per-octave amplitudes, base frequency,
world offset, iso level) so that the mean vertex height of each xy column
matches a target heightmap.  The forward keeps per-cell case indices and one
edge id per vertex; the backward recomputes the noise and its derivatives.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import abi
from .abi import check, lib
from .chunk import Context, DeviceArray, make_descs, total_cells, total_samples, totals_status


def theta_from_params(p: abi.Params) -> np.ndarray:
    """theta of a parameter set, f32 (effective amplitudes, freq, offset, iso)."""
    K = int(p.octaves)
    amps, a = [], np.float32(p.amplitude)
    for k in range(K):
        amps.append(np.float32(p.amps[k]) if p.explicit_amps else a)
        a = np.float32(a * np.float32(p.persistence))
    return np.array(amps + [p.base_freq, *p.offset, p.iso_level], dtype=np.float32)


def params_with_theta(p: abi.Params, theta) -> abi.Params:
    """Copy of p with theta applied (amplitudes become explicit)."""
    q = p.copy()
    K = int(p.octaves)
    q.explicit_amps = 1
    for k in range(K):
        q.amps[k] = float(theta[k])
    q.base_freq = float(theta[K])
    for j in range(3):
        q.offset[j] = float(theta[K + 1 + j])
    q.iso_level = float(theta[K + 4])
    return q


class Adjoint:
    """Device buffers and calls of forward/backward over a fixed chunk batch."""

    def __init__(self, ctx: Context, descs: np.ndarray, vert_capacity: int, ind_capacity: int,
                 sample_grad: bool = False):
        self.ctx = ctx
        self.descs = np.ascontiguousarray(descs, dtype=abi.CHUNK_DESC_DTYPE)
        self.n = int(self.descs.shape[0])
        self.max_cells = int(self.descs["cells"].max())
        self.vcap, self.icap = int(vert_capacity), int(ind_capacity)
        self.ncells, self.nsamp = total_cells(self.descs), total_samples(self.descs)
        self.K = int(ctx.params.octaves)
        self.d_desc = ctx.upload(self.descs)
        self.d_rec = DeviceArray(self.n * 32)
        self.d_verts = DeviceArray(self.vcap * 24)
        self.d_inds = DeviceArray(self.icap * 4)
        self.d_edges = DeviceArray(self.vcap * 4)
        self.d_cases = DeviceArray(self.ncells)
        self.d_tot = DeviceArray(32)
        self.d_pos_grad = DeviceArray(self.vcap * 12)
        self.d_theta = DeviceArray(4 * abi.theta_count(self.K))
        self.d_sgrad = DeviceArray(self.nsamp * 4) if sample_grad else None

    def out(self) -> abi.MeshOut:
        return abi.MeshOut(self.d_verts.ptr, None, self.d_inds.ptr, self.d_cases.ptr, None, self.d_rec.ptr,
                           self.d_tot.ptr, self.vcap, self.icap, self.ncells, 0)

    # -- launches (asynchronous on the context stream) ---------------------------
    def forward(self):
        out = self.out()
        check(lib().uww_forward(self.ctx.h, C.c_void_p(self.d_desc.ptr), self.n, self.max_cells, C.byref(out),
                                C.c_void_p(self.d_edges.ptr)), "uww_forward")

    def backward(self):
        check(lib().uww_backward(self.ctx.h, C.c_void_p(self.d_desc.ptr), self.n, self.max_cells,
                                 C.c_void_p(self.d_rec.ptr), C.c_void_p(self.d_edges.ptr),
                                 C.c_void_p(self.d_pos_grad.ptr), C.c_void_p(self.d_theta.ptr),
                                 C.c_void_p(self.d_sgrad.ptr) if self.d_sgrad else None,
                                 self.nsamp if self.d_sgrad else 0), "uww_backward")

    # -- transfers -------------------------------------------------------------------
    def set_pos_grad(self, g: np.ndarray):
        g = np.ascontiguousarray(g, dtype=np.float32)
        if g.size > 3 * self.vcap:
            raise ValueError(f"{g.size} gradient entries exceed 3 x the vertex capacity {self.vcap}")
        check(lib().uww_memcpy(self.ctx.h, C.c_void_p(self.d_pos_grad.ptr), g.ctypes.data_as(C.c_void_p), g.nbytes,
                               abi.H2D), "pos_grad upload")
        self.ctx.sync()

    def totals(self) -> np.ndarray:
        return self.ctx.download(self.d_tot, (4,), np.uint64)

    def fetch_forward(self) -> dict:
        tot = self.totals()
        st = totals_status(tot)
        if st:
            raise abi.UWWError(st, "uww_forward")
        nv = int(tot[0])
        return {"totals": tot,
                "records": self.ctx.download(self.d_rec, (self.n,), abi.CHUNK_RECORD_DTYPE),
                "verts": self.ctx.download(self.d_verts, (nv,), abi.VERT_COLOR_DTYPE),
                "edge_ids": self.ctx.download(self.d_edges, (nv,), np.uint32),
                "cases": self.ctx.download(self.d_cases, (self.ncells,), np.uint8)}

    def theta_grad(self) -> np.ndarray:
        return self.ctx.download(self.d_theta, (abi.theta_count(self.K),), np.float32)

    def sample_grad(self) -> np.ndarray:
        if self.d_sgrad is None:
            raise ValueError("built without sample_grad=True")
        return self.ctx.download(self.d_sgrad, (self.nsamp,), np.float32)


# ---- terrain fitting -----------------------------------------------------------
def gaussian_heightmap(cols: int, column: float, n_bumps: int = 8, seed: int = 0, sigma=(20.0, 80.0),
                       height=(40.0, 200.0), base: float = 0.0) -> np.ndarray:
    """Seeded target: base + sum of isotropic Gaussians, centres uniform over the
    area, sigma and height uniform in the given ranges (world units); sampled
    at column centres, shape (cols, cols) indexed [cy, cx]."""
    rng = np.random.default_rng(seed)
    ext = cols * column
    c = (np.arange(cols) + 0.5) * column
    X, Y = np.meshgrid(c, c)
    hm = np.full((cols, cols), base, dtype=np.float64)
    for _ in range(n_bumps):
        cx, cy = rng.uniform(0, ext, 2)
        s = rng.uniform(*sigma)
        h = rng.uniform(*height)
        hm += h * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    return hm.astype(np.float32)


class TerrainFit:
    """Adam on theta so that each xy column's mean vertex z matches a heightmap.

    One step: forward (build + edge ids), heightmap loss and dL/dp on the
    device, backward (dL/dtheta), then the Adam update on the host.  Adam runs
    on phi with theta = theta0 + scale * phi, one scale per entry so that a unit
    of phi is a comparable change: the initial value for the amplitudes and the
    frequency (relative steps), one noise period 1 / f0 for the offsets, and
    the density change that moves a linear-bias surface across `height` world
    units for the iso level.  If the mesh outgrows the vertex or index
    capacity, the buffers are doubled and the step is repeated.
    """

    def __init__(self, ctx: Context, descs: np.ndarray, target: np.ndarray, column: float, origin=(0.0, 0.0),
                 vert_capacity: int = 1 << 22, ind_capacity: int = 1 << 24, lr: float = 1e-2,
                 height: float | None = None):
        self.ctx = ctx
        self.base = ctx.params.copy()
        self.descs = descs
        self.adj = Adjoint(ctx, descs, vert_capacity, ind_capacity)
        self.cols_y, self.cols_x = target.shape
        self.column = float(column)
        self.origin = origin
        self.d_target = ctx.upload(np.ascontiguousarray(target, dtype=np.float32))
        self.d_work = DeviceArray(4 * target.size * 4)
        self.d_loss = DeviceArray(4)
        self.theta0 = theta_from_params(ctx.params).astype(np.float64)
        K = int(ctx.params.octaves)
        f0 = float(self.theta0[K])
        if height is None:
            zs = descs["pos"][:, 2].astype(np.float64) * ctx.params.chunk_size
            height = float(zs.max() - zs.min() + ctx.params.chunk_size)
        slope = abs(ctx.params.bias_a) if ctx.params.bias_mode == abi.UWW_BIAS_LINEAR else 1.0
        self.scale = np.concatenate([np.abs(self.theta0[:K]), [f0], np.full(3, 1.0 / f0), [slope * height]])
        self.scale[self.scale == 0] = 1.0
        self.phi = np.zeros_like(self.theta0)
        self.lr = lr
        self.m = np.zeros_like(self.phi)
        self.v = np.zeros_like(self.phi)
        self.t = 0

    @property
    def theta(self) -> np.ndarray:
        return self.theta0 + self.scale * self.phi

    def _evaluate(self):
        a = self.adj
        self.ctx.set_params(params_with_theta(self.base, self.theta))
        a.forward()
        check(lib().uww_height_loss(self.ctx.h, C.c_void_p(a.d_verts.ptr), C.c_void_p(a.d_tot.ptr), a.vcap,
                                    self.origin[0], self.origin[1], self.column, self.cols_x, self.cols_y,
                                    C.c_void_p(self.d_target.ptr), C.c_void_p(self.d_work.ptr),
                                    C.c_void_p(a.d_pos_grad.ptr), C.c_void_p(self.d_loss.ptr)), "uww_height_loss")
        a.backward()
        g = a.theta_grad().astype(np.float64)        # synchronises
        loss = float(self.ctx.download(self.d_loss, (1,), np.float32)[0])
        return loss, g, a.totals()

    def step(self) -> tuple[float, np.ndarray]:
        for _ in range(8):
            loss, g, tot = self._evaluate()
            st = totals_status(tot)
            if st == abi.UWW_OK:
                break
            if st != abi.UWW_ERR_CAPACITY:
                raise abi.UWWError(st, "terrain fit forward")
            a = self.adj
            self.adj = Adjoint(self.ctx, self.descs, max(2 * a.vcap, int(tot[0]) + 1),
                               max(2 * a.icap, int(tot[1]) + 1))
        else:
            raise abi.UWWError(abi.UWW_ERR_CAPACITY, "terrain fit forward")
        # Adam (Kingma & Ba), default betas, on phi
        gp = g * self.scale
        self.t += 1
        b1, b2, eps = 0.9, 0.999, 1e-8
        self.m = b1 * self.m + (1 - b1) * gp
        self.v = b2 * self.v + (1 - b2) * gp * gp
        mh = self.m / (1 - b1 ** self.t)
        vh = self.v / (1 - b2 ** self.t)
        self.phi = self.phi - self.lr * mh / (np.sqrt(vh) + eps)
        self.last_grad = g
        return loss, g

    # ---- checkpoint / resume ---------------------------------------------------
    # A chunk's mesh is a function of (parameters, seed, position) alone -- the
    # reference regenerates chunks from them (world.rs:236-247) -- so the fit's
    # whole state is theta's parametrisation and Adam's moments.
    def state_dict(self) -> dict:
        """Everything a resumed fit needs: theta0, the per-entry scales, phi,
        Adam's moments and step count, the learning rate."""
        return {"theta0": self.theta0.copy(), "scale": self.scale.copy(), "phi": self.phi.copy(),
                "m": self.m.copy(), "v": self.v.copy(), "t": np.int64(self.t), "lr": np.float64(self.lr)}

    def load_state_dict(self, st: dict) -> None:
        theta0 = np.asarray(st["theta0"], np.float64)
        if theta0.shape != self.theta0.shape:
            raise ValueError(f"checkpoint has {theta0.size} parameters, this fit {self.theta0.size}")
        self.theta0 = theta0.copy()
        self.scale = np.asarray(st["scale"], np.float64).copy()
        self.phi = np.asarray(st["phi"], np.float64).copy()
        self.m = np.asarray(st["m"], np.float64).copy()
        self.v = np.asarray(st["v"], np.float64).copy()
        self.t = int(st["t"])
        self.lr = float(st["lr"])

    def save(self, path) -> None:
        """Write the state to an .npz file (atomically: a temporary file, then a rename)."""
        import os
        tmp = f"{path}.tmp.npz"
        np.savez(tmp, **self.state_dict())
        os.replace(tmp, path)

    def load(self, path) -> None:
        with np.load(path) as z:
            self.load_state_dict({k: z[k] for k in z.files})

    def run(self, steps: int, checkpoint=None, every: int = 0) -> dict:
        """`steps` Adam steps; with `checkpoint` (a path) and `every` > 0 the
        state is saved after every `every` steps and after the last one."""
        losses = []
        t0 = time.perf_counter()
        for k in range(steps):
            loss, _ = self.step()
            losses.append(loss)
            if checkpoint is not None and every > 0 and ((k + 1) % every == 0 or k + 1 == steps):
                self.save(checkpoint)
        el = time.perf_counter() - t0
        g = getattr(self, "last_grad", None)
        return {"losses": losses, "seconds": el, "theta": self.theta.copy(),
                "grad_norm": float(np.linalg.norm(g)) if g is not None else None,
                "scaled_grad_norm": float(np.linalg.norm(g * self.scale)) if g is not None else None}


def terrain_volume(chunks_per_edge: int = 32, cells: int = 16, chunk_size: int = 16, octaves: int = 8, seed: int = 0,
                   slope: float | None = None):
    """The fitting volume: chunks_per_edge^3 chunks of cells^3 cells, fBm with a
    linear depth bias, so the surface lies near half the volume height and
    moves by fBm / slope (default slope 3 / height); base frequency 2 / height,
    so the eighth octave has a quarter period per cell of a 16^3-cell chunk."""
    height = chunks_per_edge * chunk_size
    p = abi.reference_params()
    p.seed = seed
    p.octaves = octaves
    p.chunk_size = chunk_size
    p.base_freq = 2.0 / height
    p.lacunarity, p.persistence, p.amplitude = 2.0, 0.5, 1.0
    p.normalize = 1
    p.bias_mode = abi.UWW_BIAS_LINEAR
    p.bias_a = slope if slope is not None else 3.0 / height
    p.bias_b = 0.5 * height
    p.iso_level = 0.0
    p.math_mode = abi.UWW_MATH_FAST
    p.dedup_mode = abi.UWW_DEDUP_EDGE
    p.outputs = abi.UWW_OUT_CASES
    r = np.arange(chunks_per_edge)
    X, Y, Z = np.meshgrid(r, r, r, indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.int32)
    return p, make_descs(pos, np.full(len(pos), cells, np.uint32))
