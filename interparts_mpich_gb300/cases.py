"""Seeded synthetic cases of the IBM channel / settling runs.

No dataset is involved in the reference's benchmarks; every input here is
generated from a seed:
  * the Lagrangian force-point table (the reference reads one produced by
    its poslfp electrostatic-repulsion generator, coordsfp.f90:21-29) is
    replaced by a deterministic Fibonacci sphere of the same size nl;
  * fields follow the reference's initial conditions ('poi' Poiseuille
    with streamwise y, init.f90:436-450; 'pur' rest, init.f90:314-328) plus,
    for the channel, seeded uniform perturbations;
  * sphere centres are drawn uniformly with rejection of gaps < 0.1 D to
    each other (periodic in x, y) and to the walls.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from ._abi import IBM_BC_FREESLIP, IBM_BC_NOSLIP, IBM_BC_PERIODIC, IBM_MODE_PLAIN_FP64, IbmParams, ParticleState, dptr


def derived_nl(radius: float, dxi: float) -> int:
    """nl = nint(pi/3 * (12*((radius-retrac)*dxi)**2 + 1)), retrac = 0.3/dxi (init.f90:127-129)."""
    retrac = 0.3 / dxi
    x = (math.pi / 3.0) * (12.0 * ((radius - retrac) * dxi) ** 2 + 1.0)
    return int(math.floor(x + 0.5))


def fibonacci_sphere(nl: int) -> tuple[np.ndarray, np.ndarray]:
    """(theta, phi) of nl nearly uniform points on the unit sphere."""
    l = np.arange(nl, dtype=np.float64)
    z = 1.0 - (2.0 * l + 1.0) / nl
    theta = np.arccos(z)
    phi = np.mod(l * math.pi * (3.0 - math.sqrt(5.0)), 2.0 * math.pi)
    return theta, phi


def bounduvw(u, v, w, bc_top=IBM_BC_NOSLIP, bc_bot=IBM_BC_NOSLIP):
    """Reference ghost values (bound.f90:11-80) on (0:i1,0:j1,0:k1) arrays;
    with IBM_BC_PERIODIC the z ghost planes are periodic copies."""
    if bc_top == IBM_BC_PERIODIC:
        for f in (u, v, w):
            f[:, :, -1] = f[:, :, 1]
            f[:, :, 0] = f[:, :, -2]
    else:
        s_top = -1.0 if bc_top == IBM_BC_NOSLIP else 1.0
        s_bot = -1.0 if bc_bot == IBM_BC_NOSLIP else 1.0
        u[:, :, -1] = s_top * u[:, :, -2]
        v[:, :, -1] = s_top * v[:, :, -2]
        w[:, :, -2] = 0.0
        u[:, :, 0] = s_bot * u[:, :, 1]
        v[:, :, 0] = s_bot * v[:, :, 1]
        w[:, :, 0] = 0.0
    for f in (u, v, w):
        f[-1, :, :] = f[1, :, :]
        f[0, :, :] = f[-2, :, :]
        f[:, -1, :] = f[:, 1, :]
        f[:, 0, :] = f[:, -2, :]


def boundp(p):
    """Reference ghost values of the pressure (boundp, bound.f90:82-107):
    Neumann at the walls, periodic in x and y, on a (0:i1,0:j1,0:k1) array."""
    p[:, :, 0] = p[:, :, 1]
    p[:, :, -1] = p[:, :, -2]
    p[-1, :, :] = p[1, :, :]
    p[0, :, :] = p[-2, :, :]
    p[:, -1, :] = p[:, 1, :]
    p[:, 0, :] = p[:, -2, :]


@dataclass
class Case:
    name: str
    itot: int
    jtot: int
    ktot: int
    lx: float = 1.0
    ly: float = 1.0
    lz: float = 1.0
    visc: float = 1.0 / 5600.0
    radius: float = 1.0 / 32.0
    ratiorho: float = 1.0
    bc_top: int = IBM_BC_NOSLIP
    bc_bot: int = IBM_BC_NOSLIP
    np: int = 0
    seed: int = 1234
    flow: str = "poi"            # 'poi' (perturbed Poiseuille) or 'pur' (rest)
    perturb: float = 0.05        # amplitude of the uniform velocity noise
    gap: float = 0.1             # minimum gap in diameters (sphere-sphere, sphere-wall)
    nb_copies: int = 9
    rotation: int = 0
    centres: np.ndarray | None = None
    velocities: np.ndarray | None = None
    radii: np.ndarray | None = None  # polydisperse: [np] radii (radius is then unused)
    _keep: list = field(default_factory=list, repr=False)

    @property
    def dxi(self) -> float:
        return self.itot / self.lx

    @property
    def nl(self) -> int:
        """Points per sphere (the largest sphere's when polydisperse)."""
        if self.np == 0:
            return 0
        if self.radii is not None:
            return max(derived_nl(float(r), self.dxi) for r in self.radii)
        return derived_nl(self.radius, self.dxi)

    @property
    def rmax(self) -> float:
        return float(np.max(self.radii)) if self.radii is not None else self.radius

    @property
    def nq(self) -> int:
        return min(self.np + 2, 15)

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.itot + 2, self.jtot + 2, self.ktot + 2)

    def lagrangian_table(self):
        """(theta, phi, radfp); polydisperse: every sphere's table of its own
        point count, one after the other (radfp unused)."""
        nl = self.nl
        if nl == 0:
            return np.zeros(1), np.zeros(1), 0.0
        if self.radii is not None:
            tabs = [fibonacci_sphere(derived_nl(float(r), self.dxi)) for r in self.radii]
            return (np.ascontiguousarray(np.concatenate([t[0] for t in tabs])),
                    np.ascontiguousarray(np.concatenate([t[1] for t in tabs])), self.rmax - 0.3 / self.dxi)
        theta, phi = fibonacci_sphere(nl)
        radfp = self.radius - 0.3 / self.dxi
        return theta, phi, radfp

    def params(self, mode: int = IBM_MODE_PLAIN_FP64) -> IbmParams:
        theta, phi, radfp = self.lagrangian_table()
        radii = None if self.radii is None else np.ascontiguousarray(self.radii, dtype=np.float64)
        self._keep = [theta, phi, radii]
        return IbmParams(
            itot=self.itot, jtot=self.jtot, ktot=self.ktot, lx=self.lx, ly=self.ly, lz=self.lz,
            visc=self.visc, radius=self.radius, ratiorho=self.ratiorho,
            bc_top=self.bc_top, bc_bot=self.bc_bot, particle_rotation=self.rotation,
            np=self.np, nl=self.nl, thetarc=dptr(theta), phirc=dptr(phi), radfp=radfp,
            nb_copies=self.nb_copies, mode=mode, radii=dptr(radii) if radii is not None else None)

    # ---- fields -----------------------------------------------------------
    def initial_fields(self) -> dict[str, np.ndarray]:
        shp = self.shape
        u = np.zeros(shp, order="F")
        v = np.zeros(shp, order="F")
        w = np.zeros(shp, order="F")
        p = np.zeros(shp, order="F")
        if self.flow == "poi":
            dz = self.lz / self.ktot
            k = np.arange(self.ktot + 2, dtype=np.float64)
            coorz = (k - 0.5) * dz / self.lz
            v[:, :, :] = (6.0 * 1.0 * coorz * (1.0 - coorz))[None, None, :]
        if self.perturb > 0 and self.flow == "poi":
            rng = np.random.default_rng(self.seed)
            n = (self.itot, self.jtot, self.ktot)
            for f in (u, v, w):
                f[1:-1, 1:-1, 1:-1] += rng.uniform(-self.perturb, self.perturb, n).astype(np.float64)
        bounduvw(u, v, w, self.bc_top, self.bc_bot)
        return {"u": u, "v": v, "w": w, "p": p}

    # ---- particles ----------------------------------------------------------
    def sphere_centres(self) -> np.ndarray:
        if self.centres is not None:
            return np.asarray(self.centres, np.float64).reshape(self.np, 3)
        if getattr(self, "_placed", None) is None:
            self._placed = self._place_spheres()
        return self._placed.copy()

    def _place_spheres(self) -> np.ndarray:
        """Seeded uniform centres with rejection of gaps below gap x the
        diameter (gap x the mean of the two diameters between unequal
        spheres) to each other and to the walls."""
        radii = (np.asarray(self.radii, np.float64) if self.radii is not None
                 else np.full(self.np, self.radius))
        R = float(radii.max())
        D = 2 * R
        dmin = D + self.gap * D  # the largest pair distance tested: cell size
        rng = np.random.default_rng(self.seed + 7919)
        out = np.zeros((self.np, 3))
        # accepted centres binned in cells at least dmin wide (periodic in x
        # and y): a candidate is tested against the spheres of its 27
        # neighbouring cells only, which are all that can lie within dmin
        nx = max(1, int(self.lx // dmin))
        ny = max(1, int(self.ly // dmin))
        nz = max(1, int(self.lz // dmin))
        cells: dict[tuple[int, int, int], list[int]] = {}

        def cell(c):
            return (min(int(c[0] / self.lx * nx), nx - 1), min(int(c[1] / self.ly * ny), ny - 1),
                    min(int(c[2] / self.lz * nz), nz - 1))

        n = 0
        tries = 0
        while n < self.np:
            tries += 1
            if tries > 2000 * max(1, self.np):
                raise RuntimeError("could not place the spheres without overlap")
            rn = radii[n]
            if self.radii is None:
                zlo, zhi = rn + self.gap * D, self.lz - rn - self.gap * D
            else:
                zlo, zhi = rn * (1 + 2 * self.gap), self.lz - rn * (1 + 2 * self.gap)
            c = np.array([rng.uniform(0, self.lx), rng.uniform(0, self.ly), rng.uniform(zlo, zhi)])
            if n:
                ix, iy, iz = cell(c)
                near = []
                for a in {(ix + q) % nx for q in (-1, 0, 1)}:
                    for b in {(iy + q) % ny for q in (-1, 0, 1)}:
                        for z in range(max(iz - 1, 0), min(iz + 2, nz)):
                            near.extend(cells.get((a, b, z), ()))
                if near:
                    d = np.abs(out[near] - c)
                    d[:, 0] = np.minimum(d[:, 0], self.lx - d[:, 0])
                    d[:, 1] = np.minimum(d[:, 1], self.ly - d[:, 1])
                    d2 = np.sum(d * d, axis=1)
                    if self.radii is None:
                        if np.min(d2) < dmin * dmin:
                            continue
                    else:
                        lim = (radii[near] + rn) * (1 + self.gap)
                        if np.any(d2 < lim * lim):
                            continue
            out[n] = c
            cells.setdefault(cell(c), []).append(n)
            n += 1
        return out

    def initial_particles(self, lagrangian: bool = True) -> ParticleState:
        ps = ParticleState(self.np, self.nq, self.nl, lagrangian=lagrangian)
        if self.np:
            c = self.sphere_centres()
            ps.x[:], ps.y[:], ps.z[:] = c[:, 0], c[:, 1], c[:, 2]
            if self.velocities is not None:
                vel = np.asarray(self.velocities, np.float64).reshape(self.np, 3)
                ps.u[:], ps.v[:], ps.w[:] = vel[:, 0], vel[:, 1], vel[:, 2]
        return ps


# ---- the benchmark configurations -------------------------------------------------
def channel_case(n: int = 256, nspheres: int = 1000, seed: int = 1234) -> Case:
    """Dense suspension in a channel: n^3 grid, walls at z=0 and z=1, perturbed
    Poiseuille flow at bulk Re 5600 (streamwise y), neutrally buoyant spheres of
    D = 16 dx with gaps >= 0.1 D."""
    return Case(name=f"channel{n}_np{nspheres}", itot=n, jtot=n, ktot=n, visc=1.0 / 5600.0,
                radius=8.0 / n, ratiorho=1.0, np=nspheres, seed=seed, flow="poi", perturb=0.05)


def wide_channel_case(nx: int = 512, nz: int = 256, nspheres: int = 8000, seed: int = 1234) -> Case:
    """The wide channel of the learned-forcing runs: nx x nx x nz grid on a
    (2, 2, 1) box (dx = 1/nz), walls at z = 0 and z = 1, perturbed Poiseuille
    flow at bulk Re 5600 (streamwise y), neutrally buoyant spheres of
    D = 16 dx placed at random without overlap (gaps >= 0.05 D to each other
    and to the walls; at 8000 spheres the volume fraction is 25.6 %)."""
    lx = nx / nz
    return Case(name=f"wide{nx}x{nz}_np{nspheres}", itot=nx, jtot=nx, ktot=nz, lx=lx, ly=lx, lz=1.0,
                visc=1.0 / 5600.0, radius=8.0 / nz, ratiorho=1.0, np=nspheres, seed=seed, flow="poi", perturb=0.05,
                gap=0.05)


def settling_case(n: int = 64, seed: int = 1, periodic: bool = True) -> Case:
    """Single settling sphere D = 16 dx at the centre of the unit cube,
    density ratio 1.5, Galileo 150 (nu = sqrt((rho_r - 1) g D^3) / Ga),
    fluid at rest.  periodic: triply periodic (IBM_BC_PERIODIC in z, a
    variant of the method the reference, with walls in z, cannot express);
    otherwise free-slip walls in z."""
    R = 8.0 / n
    D = 2 * R
    ga = 150.0
    visc = math.sqrt((1.5 - 1.0) * 9.81 * D ** 3) / ga
    bc = IBM_BC_PERIODIC if periodic else IBM_BC_FREESLIP
    return Case(name=f"settling{n}{'p' if periodic else 'w'}", itot=n, jtot=n, ktot=n, visc=visc, radius=R,
                ratiorho=1.5, bc_top=bc, bc_bot=bc, np=1, seed=seed, flow="pur", perturb=0.0,
                centres=np.array([[0.5, 0.5, 0.5]]))


def poly_case(nx: int = 768, nz: int = 384, nspheres: int = 15000, seed: int = 1234, dmin_cells: float = 12.0,
              dmax_cells: float = 24.0) -> Case:
    """Polydisperse settling suspension: nx x nx x nz grid on a (nx/nz,
    nx/nz, 1) box (dx = 1/nz), periodic in x and y, no-slip walls in z; spheres
    with D drawn uniformly from [dmin, dmax] dx (seeded), placed at random
    without overlap (gaps >= 0.05 D); density ratio 2.0, gravity in -z,
    Galileo number 200 on the mean diameter (nu = sqrt((rho_r - 1) g D^3) /
    Ga); fluid at rest.  At 768 x 768 x 384 with 15000 spheres of 12..24 dx
    the solid volume fraction is about 22 %."""
    lx = nx / nz
    dx = 1.0 / nz
    rng = np.random.default_rng(seed + 104729)
    radii = 0.5 * dx * rng.uniform(dmin_cells, dmax_cells, nspheres)
    dmean = 0.5 * (dmin_cells + dmax_cells) * dx
    visc = math.sqrt((2.0 - 1.0) * 9.81 * dmean ** 3) / 200.0
    return Case(name=f"poly{nx}x{nz}_np{nspheres}", itot=nx, jtot=nx, ktot=nz, lx=lx, ly=lx, lz=1.0, visc=visc,
                radius=float(radii.max()), ratiorho=2.0, np=nspheres, seed=seed, flow="pur", perturb=0.0, gap=0.05,
                radii=radii)
