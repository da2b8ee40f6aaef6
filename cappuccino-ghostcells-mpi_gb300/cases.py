"""Synthetic cases with the shapes of the benchmarked configurations.

The reference reads its grid from an unformatted file written by a grid
generator that is not part of the repository (read_grid.f90:126-161), and
perturbs its initial field from /dev/urandom (random_seed.f90:11-14).
This module is the build's own generator: seeded, reproducible, and
writing exactly the module arrays that read_grid/init fill in.

Storage follows setind.f90:34-40: a field of an ni x nj x nk grid is a flat
array with j fastest, then i, then k (numpy shape (nk, ni, nj), C order).
N interior cells per axis means ni = N + 4: layers 2 and N+3 are ghost
cells, layers 1 and N+4 are padding.  Node (i,j,k) is the east-north-top
corner of cell (i,j,k) (init.f90:54-73), so the physical nodes are node
indices 2..N+2.

Quantities read from the grid file (x, y, z, xc, yc, zc, vol) are produced
here; face areas and interpolation factors are recomputed from the nodes
by the library exactly as init.f90:54-144 does.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from .params import IU, IV, IW, IP, ITE, IED, IVIS, SOLVER, NPHI

DEFAULT_SEED = 20261203


@dataclass
class Case:
    name: str
    ni: int
    nj: int
    nk: int
    fields: dict = field(default_factory=dict)   # name -> float64 (nk*ni*nj,)
    bc: dict = field(default_factory=dict)       # lbw..lbt -> int32 arrays
    params: dict = field(default_factory=dict)   # cappgpu_params members
    meta: dict = field(default_factory=dict)

    @property
    def nijk(self):
        return self.ni * self.nj * self.nk

    @property
    def interior(self):
        return (self.ni - 4, self.nj - 4, self.nk - 4)

    def view(self, a):
        """(k, i, j) view of a flat field, 0-based indices = reference index - 1."""
        return np.asarray(a).reshape(self.nk, self.ni, self.nj)

    def ijk(self, i, j, k):
        """0-based storage index of the reference's ijk = lk(k)+li(i)+j."""
        return (k - 1) * self.ni * self.nj + (i - 1) * self.nj + (j - 1)


# ------------------------------------------------------------------ grids

def _pad_nodes(p):
    """Extend physical nodes (Ni+1, Nj+1, Nk+1, 3) by linear extrapolation:
    2 layers low (node index 0 and 1) and 2 high (nim, ni)."""
    return np.pad(p, ((2, 2), (2, 2), (2, 2), (0, 0)), mode="reflect", reflect_type="odd")


def _hex_volume(q):
    """Volume of every cell from padded nodes q (indices 0..ni per axis):
    sum over the six faces of (face centre . outward area) / 3, with the
    face area vectors of init.f90:54-136 (half the diagonal cross product)."""
    def area(a, b, c, d):
        # face nodes a=inp, b=ins, c=inb, d=inbs as in init.f90
        dxet = 0.5 * (a - b + c - d)
        dxzd = 0.5 * (a - c + b - d)
        return np.stack([dxet[..., 1] * dxzd[..., 2] - dxzd[..., 1] * dxet[..., 2],
                         dxzd[..., 0] * dxet[..., 2] - dxet[..., 0] * dxzd[..., 2],
                         dxet[..., 0] * dxzd[..., 1] - dxet[..., 1] * dxzd[..., 0]], axis=-1)

    def centre(a, b, c, d):
        return 0.25 * (a + b + c + d)

    # node q[i, j, k]; cell (i,j,k) for i,j,k = 1..ni spans nodes i-1..i
    n000 = q[:-1, :-1, :-1]; n100 = q[1:, :-1, :-1]; n010 = q[:-1, 1:, :-1]; n110 = q[1:, 1:, :-1]
    n001 = q[:-1, :-1, 1:]; n101 = q[1:, :-1, 1:]; n011 = q[:-1, 1:, 1:]; n111 = q[1:, 1:, 1:]
    # east face (i): nodes (i,j,k),(i,j-1,k),(i,j,k-1),(i,j-1,k-1) ; west = same at i-1
    ae = area(n111, n101, n110, n100); ce = centre(n111, n101, n110, n100)
    aw = area(n011, n001, n010, n000); cw = centre(n011, n001, n010, n000)
    # north face (j): idns = nj (i direction), idtb = nij
    an = area(n111, n011, n110, n010); cn = centre(n111, n011, n110, n010)
    as_ = area(n101, n001, n100, n000); cs = centre(n101, n001, n100, n000)
    # top face (k): idns = 1 (j), idtb = nj (i)
    at = area(n111, n101, n011, n001); ct = centre(n111, n101, n011, n001)
    ab = area(n110, n100, n010, n000); cb = centre(n110, n100, n010, n000)
    # init.f90's cross products point east faces to +i but north and top
    # faces to -j and -k on a right-handed grid: flip those two terms
    vol = ((np.sum(ce * ae, -1) - np.sum(cw * aw, -1)) - (np.sum(cn * an, -1) - np.sum(cs * as_, -1))
           - (np.sum(ct * at, -1) - np.sum(cb * ab, -1))) / 3.0
    return np.abs(vol)


def build_grid(xn, yn, zn):
    """Grid arrays from physical node coordinates.

    xn, yn, zn: arrays of shape (Ni+1, Nj+1, Nk+1) indexed [i, j, k].
    Returns (ni, nj, nk, dict of flat fields x,y,z,xc,yc,zc,vol)."""
    Ni, Nj, Nk = (s - 1 for s in xn.shape)
    ni, nj, nk = Ni + 4, Nj + 4, Nk + 4
    q = _pad_nodes(np.stack([xn, yn, zn], axis=-1).astype(np.float64))  # (ni+1,)^3 nodes 0..ni
    nodes = q[1:, 1:, 1:]                                                  # reference nodes 1..ni
    cen = 0.125 * (q[:-1, :-1, :-1] + q[1:, :-1, :-1] + q[:-1, 1:, :-1] + q[1:, 1:, :-1]
                   + q[:-1, :-1, 1:] + q[1:, :-1, 1:] + q[:-1, 1:, 1:] + q[1:, 1:, 1:])
    vol = _hex_volume(q)

    def flat(a):  # [i, j, k] -> flat j-fastest, then i, then k
        return np.ascontiguousarray(np.transpose(a, (2, 0, 1))).reshape(-1)

    out = {
        "x": flat(nodes[..., 0]), "y": flat(nodes[..., 1]), "z": flat(nodes[..., 2]),
        "xc": flat(cen[..., 0]), "yc": flat(cen[..., 1]), "zc": flat(cen[..., 2]),
        "vol": flat(vol),
    }
    return ni, nj, nk, out


def uniform_nodes(N, L):
    axes = [np.linspace(0.0, L[a], N[a] + 1) for a in range(3)]
    return np.meshgrid(*axes, indexing="ij")


def channel_nodes(N, L, beta):
    """x uniform over L[0], y uniform over L[1], wall-normal z (reference k)
    with tanh stretching z = tanh(beta (2 eta - 1)) / tanh(beta) over [-1,1]
    scaled to L[2]/2."""
    x = np.linspace(0.0, L[0], N[0] + 1)
    y = np.linspace(0.0, L[1], N[1] + 1)
    eta = np.linspace(0.0, 1.0, N[2] + 1)
    z = 0.5 * L[2] * np.tanh(beta * (2.0 * eta - 1.0)) / math.tanh(beta)
    return np.meshgrid(x, y, z, indexing="ij")


def skewed_nodes(N, L, amp=0.1, seed=DEFAULT_SEED):
    """Uniform nodes displaced per axis by amp*h*sin(2 pi (k1 s + k2 t) + phi),
    tapered to zero on the boundary planes of that axis so the domain stays
    a box."""
    rng = np.random.default_rng(seed)
    X, Y, Z = uniform_nodes(N, L)
    h = [L[a] / N[a] for a in range(3)]
    S = [X / L[0], Y / L[1], Z / L[2]]
    out = []
    for a, C in enumerate((X, Y, Z)):
        b, c = [q for q in range(3) if q != a]
        k1, k2 = rng.integers(1, 4, size=2)
        phi = rng.uniform(0, 2 * math.pi)
        taper = np.sin(math.pi * S[a])
        out.append(C + amp * h[a] * taper * np.sin(2 * math.pi * (k1 * S[b] + k2 * S[c]) + phi))
    return out


# ---------------------------------------------------------------- helpers

def _bc_arrays(ni, nj, nk, codes):
    """codes: dict face -> int; arrays sized as read_grid.f90:137-139."""
    return {
        "lbw": np.full(nj * nk, codes.get("lbw", 4), np.int32),
        "lbe": np.full(nj * nk, codes.get("lbe", 4), np.int32),
        "lbs": np.full(ni * nk, codes.get("lbs", 4), np.int32),
        "lbn": np.full(ni * nk, codes.get("lbn", 4), np.int32),
        "lbb": np.full(ni * nj, codes.get("lbb", 4), np.int32),
        "lbt": np.full(ni * nj, codes.get("lbt", 4), np.int32),
    }


def _base_params():
    p = dict(alfa=0.92, densit=1.0, viscos=1e-3, timestep=1.0, btime=0.0, time=0.0,
             uin=0.0, vin=0.0, win=0.0, tein=0.0, edin=1.0, tin=0.0, flowin=0.0, zero=0.0,
             cappa=0.41, elog=8.432, gradpcmf=0.0, gravx=0.0, gravy=0.0, gravz=0.0,
             beta=0.0, tref=0.0, conumfixvalue=0.5,
             sor=[0.2] * NPHI, resor=[0.0] * NPHI, snorin=[0.0] * NPHI,
             urf=[1.0] * NPHI, gds=[1.0] * NPHI, nsw=[5] * NPHI, lcal=[0] * NPHI,
             ipr=3, jpr=3, kpr=3, ncorr=1, npcor=1, icorr=0, ipcorr=0, bdf=0, cn=0,
             lcds=1, lluds=0, lquds=0, lsmart=0, lavl=0, lmuscl=0, lumist=0, lgamma=0, lcds4=0,
             flux_limiter=0, const_mflux=0, lbuoy=0, boussinesq=0, lout=0, ltransient=0, lles=0,
             low=0, loe=0, los=0, lon=0, lob=0, lot=0,
             periodic=0, conumfix=0, isol_p=SOLVER["cgstab_sip"], piso_solver=SOLVER["pcgsip"])
    for q in (IU, IV, IW, IP):
        p["lcal"][q - 1] = 1
    return p


def initial_face_fluxes(case):
    """Mass fluxes f1,f2,f3 = den * (u_f . S_f) with linear face interpolation.
    The reference starts from f = 0 unless it reads a restart file
    (readfiles.f90:35-70); a fixed-CFL transient start needs non-zero
    fluxes, so the build derives them from the initial velocity."""
    ni, nj, nk = case.ni, case.nj, case.nk
    F = case.fields
    u, v, w = (F[c].reshape(nk, ni, nj) for c in "uvw")
    out = {}
    for name, axis, ar, fif in (("f1", 1, "ar1", "fx"), ("f2", 2, "ar2", "fy"), ("f3", 0, "ar3", "fz")):
        f = np.zeros((nk, ni, nj))
        sl0 = [slice(None)] * 3
        sl1 = [slice(None)] * 3
        sl0[axis] = slice(0, -1)
        sl1[axis] = slice(1, None)
        lam = F[fif].reshape(nk, ni, nj)[tuple(sl0)]
        uf = [c[tuple(sl1)] * lam + c[tuple(sl0)] * (1 - lam) for c in (u, v, w)]
        S = [F[ar + c].reshape(nk, ni, nj)[tuple(sl0)] for c in "xyz"]
        f[tuple(sl0)] = case.params["densit"] * (uf[0] * S[0] + uf[1] * S[1] + uf[2] * S[2])
        out[name] = f.reshape(-1)
    return out


def _common_fields(case, nijk):
    z = np.zeros(nijk)
    for n in ("u", "v", "w", "p", "pp", "te", "ed", "t", "f1", "f2", "f3", "uo", "vo", "wo",
              "uoo", "voo", "woo", "strain"):
        case.fields.setdefault(n, z.copy())
    case.fields["den"] = np.full(nijk, case.params["densit"])  # init.f90:500-502
    vis = np.zeros((case.nk, case.ni, case.nj))
    vis[1:-1, 1:-1, 1:-1] = case.params["viscos"]              # init.f90:387-460
    case.fields["vis"] = vis.reshape(-1)
    zc = case.fields["zc"].reshape(case.nk, case.ni, case.nj)
    case.fields["walldist"] = (zc - zc[0:1]).reshape(-1)       # init.f90:561-575


# ---------------------------------------------------------------- configs

def cavity(N=32, seed=DEFAULT_SEED):
    """3-D lid-driven cavity, unit cube, N^3 uniform cells, lid u=1 on the
    top (k) boundary through the inlet-type Dirichlet ghost formula, other
    walls no-slip; Re = 1000 (nu = 1e-3); SIMPLE with urf 0.7 (u,v,w) /
    0.3 (p); sipsol (alfa = 0.92) for momentum and pcgsip for p'."""
    N3 = (N, N, N) if np.isscalar(N) else tuple(N)
    ni, nj, nk, g = build_grid(*uniform_nodes(N3, (1.0, 1.0, 1.0)))
    p = _base_params()
    p.update(viscos=1e-3, uin=1.0)
    p["urf"][IU - 1] = p["urf"][IV - 1] = p["urf"][IW - 1] = 0.7
    p["urf"][IP - 1] = 0.3
    p["sor"][IU - 1] = p["sor"][IV - 1] = p["sor"][IW - 1] = 0.2
    p["nsw"][IU - 1] = p["nsw"][IV - 1] = p["nsw"][IW - 1] = 5
    p["sor"][IP - 1] = 1e-6
    p["nsw"][IP - 1] = 400
    p["isol_p"] = SOLVER["pcgsip"]
    case = Case("cavity", ni, nj, nk, fields=dict(g), params=p)
    case.bc = _bc_arrays(ni, nj, nk, {"lbt": 1})
    _common_fields(case, ni * nj * nk)
    case.meta.update(config="3D lid-driven cavity, SIMPLE", N=N3, seed=seed)
    return case


def channel(N=(128, 128, 128), beta=2.0, seed=DEFAULT_SEED, L=(2 * math.pi, math.pi, 2.0)):
    """Channel: N cells over 2pi (x, reference i) x pi (spanwise y,
    reference j) x 2 (wall-normal, reference k: the reference hard-wires the
    walls to k, calcuvw.f90:161-337); periodic in i and j
    (update_values_at_ghostcells.f90); tanh wall stretching beta = 2;
    nu = 1/180; Poiseuille u = 1.5 (1 - z^2) plus a seeded uniform
    perturbation of 10% of the centreline velocity on u, v, w; PISO with 2
    correctors, fixed CFL 0.5 (CourantNo.h:58-64); Smagorinsky LES
    (lles, lcal(ivis): calc_vis_les.f90, whose coefficient is 0.17 with Van
    Driest damping, the strain from find_strain_rate.f90); constant mass
    flux at the bulk velocity uin = 1 of the Poiseuille profile
    (const_massflux_correction.f90, the source gradpcmf*vol of
    calcuvw.f90:78)."""
    N3 = tuple(N) if not np.isscalar(N) else (N, N, N)
    ni, nj, nk, g = build_grid(*channel_nodes(N3, L, beta))
    p = _base_params()
    # alfa: init.f90:164 hard-codes ALFA = 0.92 for every SIP use.  On this
    # tanh-stretched channel PCG-SIP with 0.92 stalls above the 1e-6 target
    # (the SIP preconditioner is not symmetric); 0.5 converges (about 140
    # iterations at 128^3).  Same code path, different module value.
    p.update(viscos=1.0 / 180.0, ltransient=1, bdf=1, btime=0.0, periodic=1, ncorr=2, npcor=1,
             conumfix=1, conumfixvalue=0.5, timestep=1e-3, alfa=0.5, lles=1, const_mflux=1, uin=1.0)
    p["lcal"][IVIS - 1] = 1
    p["sor"][IU - 1] = p["sor"][IV - 1] = p["sor"][IW - 1] = 1e-3
    p["nsw"][IU - 1] = p["nsw"][IV - 1] = p["nsw"][IW - 1] = 20
    p["sor"][IP - 1] = 1e-6
    p["nsw"][IP - 1] = 2000
    p["ipr"], p["jpr"], p["kpr"] = 3, 3, 3 + N3[2] // 2
    case = Case("channel", ni, nj, nk, fields=dict(g), params=p)
    case.bc = _bc_arrays(ni, nj, nk, {})
    _common_fields(case, ni * nj * nk)
    rng = np.random.default_rng(seed)
    zc = case.fields["zc"].reshape(nk, ni, nj)
    ucl = 1.5
    shape = (nk, ni, nj)
    u = ucl * (1.0 - zc ** 2) + 0.1 * ucl * rng.uniform(-1, 1, shape)
    v = 0.1 * ucl * rng.uniform(-1, 1, shape)
    w = 0.1 * ucl * rng.uniform(-1, 1, shape)
    mask = np.zeros(shape, bool)
    mask[2:-2, 2:-2, 2:-2] = True
    for name, a in (("u", u), ("v", v), ("w", w)):
        a = np.where(mask, a, 0.0)
        case.fields[name] = a.reshape(-1)
    case.meta.update(config="channel, PISO", N=N3, seed=seed, beta=beta, L=L)
    return case


def rans_channel(N=(512, 256, 256), beta=2.5, L=(8 * math.pi, 2 * math.pi, 2.0), re_tau=590.0):
    """Large RANS channel: N cells over 8pi (x, reference i) x 2pi (spanwise,
    j) x 2 (wall-normal, k); periodic in i and j; tanh wall stretching
    beta = 2.5; nu = 1/590 (u_tau = 1 at Re_tau = 590); Menter's k-omega SST
    (sst, lcal of te, ed and vis; calcscm.f90, modvis.f90); initial fields:
    the log-law mean velocity u+ = ln(y+)/0.41 + 5.2 (u+ = y+ below
    y+ = 11), the log-law equilibrium k = u_tau^2/sqrt(0.09) (scaled by
    (y+/10)^2 below y+ = 10) and wall-resolved omega = u_tau/(sqrt(0.09)
    0.41 y), floored at k = 1e-3 and omega = 1, and the eddy viscosity of
    init.f90:474; PISO with 2 correctors at CFL 0.5; constant mass flux at
    the initial profile's bulk velocity; upwind convection for k and omega.
    From uniform k = 1e-3 and omega = 1 the SST path as the reference
    builds it drives k in the wall-adjacent cells below zero in the first
    step (the explicit diffusion correction at the wall face), clips it to
    small (calcscm.f90:595-599), and the omega source alphasst P / nu_t
    (calcscm.f90:425-427) is 0/0 in the next; the equilibrium profiles keep
    nu_t > 0.

    Two settings follow from the reference rather than from the model:
    cmu stays 0 (init.f90:177 assigns it for the k-epsilon models only, and
    modvis.f90:217 divides by it, so F2 = 1), and the top wall plane is
    lk(nkmm) (params.top_plane = 1): calcuvw.f90:254 writes lk(nimm), which
    lies outside the arrays for ni > nk."""
    N3 = tuple(N) if not np.isscalar(N) else (N, N, N)
    ni, nj, nk, g = build_grid(*channel_nodes(N3, L, beta))
    p = _base_params()
    viscos = 1.0 / re_tau
    p.update(viscos=viscos, ltransient=1, bdf=1, btime=0.0, periodic=1, ncorr=2, npcor=1,
             conumfix=1, conumfixvalue=0.5, timestep=1e-3, alfa=0.5, lles=0, const_mflux=1,
             sst=1, cmu=0.0, top_plane=1)
    for q in (ITE, IED, IVIS):
        p["lcal"][q - 1] = 1
    for q in (IU, IV, IW, ITE, IED):
        p["sor"][q - 1] = 1e-3
        p["nsw"][q - 1] = 20
    # upwind convection of k and omega (gds = 0: no deferred correction,
    # fluxscm-overrelaxed-correction.f90:197); with central differences k
    # undershoots, is clipped to small and omega's P / nu_t term turns 0/0
    p["gds"][ITE - 1] = p["gds"][IED - 1] = 0.0
    p["sor"][IP - 1] = 1e-6
    p["nsw"][IP - 1] = 2000
    p["ipr"], p["jpr"], p["kpr"] = 3, 3, 3 + N3[2] // 2
    case = Case("rans_channel", ni, nj, nk, fields=dict(g), params=p)
    case.bc = _bc_arrays(ni, nj, nk, {})
    _common_fields(case, ni * nj * nk)
    shape = (nk, ni, nj)
    zc = case.fields["zc"].reshape(shape)
    yw = np.clip(1.0 - np.abs(zc), 1e-12, None)   # distance to the nearer wall
    ypl = yw * re_tau
    uplus = np.where(ypl < 11.0, ypl, np.log(np.maximum(ypl, 1.0)) / 0.41 + 5.2)
    mask = np.zeros(shape, bool)
    mask[2:-2, 2:-2, 2:-2] = True
    u = np.where(mask, uplus, 0.0)
    case.fields["u"] = u.reshape(-1)
    sqb = math.sqrt(0.09)
    k0 = np.maximum(np.minimum(1.0, (ypl / 10.0) ** 2) / sqb, 1e-3)
    w0 = np.maximum(1.0 / (sqb * 0.41 * yw), 1.0)
    case.fields["te"] = np.where(mask, k0, 0.0).reshape(-1)
    case.fields["ed"] = np.where(mask, w0, 0.0).reshape(-1)
    den = case.fields["den"]
    vis = case.fields["vis"].copy()
    inner = mask.reshape(-1)
    vis[inner] = viscos + den[inner] * case.fields["te"][inner] / (case.fields["ed"][inner] + 1e-30)   # init.f90:474
    case.fields["vis"] = vis
    # bulk velocity of the initial profile (volume-weighted), held by const_mflux
    vol = case.fields["vol"].reshape(shape)[2:-2, 2:-2, 2:-2]
    ub = float((u[2:-2, 2:-2, 2:-2] * vol).sum() / vol.sum())
    case.params["uin"] = ub
    case.meta.update(config="RANS channel, k-omega SST", N=N3, beta=beta, L=L, re_tau=re_tau)
    return case


def poisson(N=(256, 256, 256), amp=0.1, seed=DEFAULT_SEED):
    """Skewed-grid pressure-correction system: uniform unit-cube nodes
    displaced by seeded sinusoids of amplitude amp*h per axis.  The matrix
    is assembled by piso_assemble_pressure_eq with vol*apu*den = 1 (apu =
    1/vol); boundary links are removed (pure Neumann) and one reference
    cell is pinned (PISO_multiple_correction.f90:117-129).  The right-hand
    side su is the negative divergence of a seeded Gaussian face-velocity
    field, mean removed."""
    N3 = tuple(N) if not np.isscalar(N) else (N, N, N)
    ni, nj, nk, g = build_grid(*skewed_nodes(N3, (1.0, 1.0, 1.0), amp, seed))
    p = _base_params()
    p["sor"][IP - 1] = 1e-6
    p["nsw"][IP - 1] = 4000
    # PCG-SIP with the reference's ALFA = 0.92 (init.f90:164) stalls on this
    # pinned Neumann system (oracle, 16^3: relative residual 6e-3 after 4000
    # iterations), and with 0.5 from 48^3 on (1.7e-6 after 4000); SIP's
    # factors are not symmetric for alfa > 0.  With alfa = 0 (the symmetric
    # incomplete factorisation) it reaches 1e-6 in 39 / 115 / 226 iterations
    # at 16^3 / 48^3 / 96^3.
    p["alfa"] = 0.0
    case = Case("poisson", ni, nj, nk, fields=dict(g), params=p)
    case.bc = _bc_arrays(ni, nj, nk, {})
    _common_fields(case, ni * nj * nk)
    case.fields["apu"] = 1.0 / case.fields["vol"]
    rng = np.random.default_rng(seed + 1)
    shape = (nk, ni, nj)
    for c in "uvw":
        case.fields[c] = rng.standard_normal(shape).reshape(-1)
    case.meta.update(config="skewed Poisson", N=N3, seed=seed, amp=amp)
    return case


def finalize_case(case):
    """Steps that need the library's geometry (face areas, interpolation
    factors): initial fluxes for the transient cases."""
    if case.name in ("channel", "rans_channel"):
        case.fields.update(initial_face_fluxes(case))
    return case
