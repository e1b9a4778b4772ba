"""Seeded synthetic NICAM states and the mp_driver argument table.

The reference runs one NSW6 microphysics call on a NICAM snapshot that is not
distributed with it (run/data/*.dat, README.md:81).  This module generates
physically plausible stand-in states with the shapes and value distributions
of the benchmark workloads:

* vertical grid with ``kall`` levels (one halo level below and above),
  interface heights ``gzh[k] = ztop * ((k-1)/(kall-2))**1.5`` for k >= 1,
  mirrored halos following the convention of the reference's 96-level grid
  (run/data/vgrid/GRD_{gz,gzh}.dat: gzh[0] = -gzh[2], gz[0] = -gz[1],
  gz[kall-1] = 2 gzh[kall-1] - gz[kall-2]);
* temperature 300 K (260 K in the cold variant) at the surface with a
  6.5 K/km lapse rate, floored at 210 K, plus N(0, 1 K) noise; hydrostatic
  pressure from 1000 hPa; ideal-gas density;
* QV from a relative humidity drawn from U(0.6, 1.05); QC (T > 273 K) and
  QI (T < 273 K) lognormal with median 1e-5 kg/kg in 30 % of the cells;
  QR/QS/QG lognormal with median 1e-6 kg/kg in 20 % of the cells;
* horizontal wind N(0, 10 m/s) along the local east/north unit vectors,
  vertical wind N(0, 1 m/s);
* a convective variant in which 10 % of the columns are saturated up to
  10 km and carry rain up to 5e-3 kg/kg, so that the sedimentation departure
  distance spans more than one layer.

The metric factors are those of a spherical shell, gsgam2 = gam2 =
(1 + z/a)^2 with a = 6.37122e6 m (a generator choice: the benchmark leaves
them open).  All arrays are float64 in the reference's C order: [k][g] per
region, tracers [nq][k][g], precipitation [2][g].
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# ---------------------------------------------------------------- constants
# Physical constants of the reference (include/problemsize.h:86-135).
GRAV = 9.79764
RDRY = 287.04
RVAP = 461.46
CVDRY = 717.56
LHV = 2501000.0
PSAT0 = 610.7
TEM00 = 273.15
EARTH_RADIUS = 6.37122e6

NQ = 6
I_QV, I_QC, I_QR, I_QI, I_QS, I_QG = range(6)

# ------------------------------------------------------- argument table
# The 50 array arguments of the reference mp_driver in their order
# (mod_mp_driver.h:71-124), with the per-region shape class and intent.
#   kg  -> [kall][gall]      qkg -> [6][kall][gall]
#   2g  -> [2][gall]         g   -> [gall]           1g -> [1][gall]
MP_DRIVER_ARGS: list[tuple[str, str, str]] = [
    ("rhog", "kg", "inout"),
    ("rhogvx", "kg", "inout"),
    ("rhogvy", "kg", "inout"),
    ("rhogvz", "kg", "inout"),
    ("rhogw", "kg", "inout"),
    ("rhoge", "kg", "inout"),
    ("rhogq", "qkg", "inout"),
    ("vx", "kg", "in"),
    ("vy", "kg", "in"),
    ("vz", "kg", "in"),
    ("w", "kg", "in"),
    ("unccn", "kg", "in"),
    ("rho", "kg", "inout"),
    ("tem", "kg", "inout"),
    ("pre", "kg", "inout"),
    ("q", "qkg", "inout"),
    ("qd", "kg", "out"),
    ("precip", "2g", "out"),
    ("ISO1_precip", "2g", "out"),
    ("ISO2_precip", "2g", "out"),
    ("precip_rhoe", "g", "out"),
    ("precip_lh_heat", "g", "out"),
    ("precip_rhophi", "g", "out"),
    ("precip_rhokin", "g", "out"),
    ("re_liquid", "kg", "out"),
    ("re_solid", "kg", "out"),
    ("re_cld", "kg", "out"),
    ("rctop", "1g", "out"),
    ("rwtop", "1g", "out"),
    ("tctop", "1g", "out"),
    ("frhoge_af", "kg", "in"),
    ("frhogqv_af", "kg", "in"),
    ("frhoge_rad", "kg", "in"),
    ("rhogqke", "kg", "in"),
    ("gsgam2", "kg", "in"),
    ("gsgam2h", "kg", "in"),
    ("gam2", "kg", "in"),
    ("gam2h", "kg", "in"),
    ("ix", "g", "in"),
    ("iy", "g", "in"),
    ("iz", "g", "in"),
    ("jx", "g", "in"),
    ("jy", "g", "in"),
    ("jz", "g", "in"),
    ("z", "kg", "in"),
    ("zh", "kg", "in"),
    ("GDCLW", "kg", "out"),
    ("GDCFRC", "kg", "out"),
    ("GPREC", "kg", "out"),
    ("CBMFX", "kg", "in"),
]
ARG_NAMES = [a[0] for a in MP_DRIVER_ARGS]
ARG_INDEX = {a[0]: i for i, a in enumerate(MP_DRIVER_ARGS)}
OUTPUT_NAMES = [n for n, _, it in MP_DRIVER_ARGS if it in ("out", "inout")]


def region_shape(kind: str, kall: int, gall: int) -> tuple[int, ...]:
    return {
        "kg": (kall, gall),
        "qkg": (NQ, kall, gall),
        "2g": (2, gall),
        "g": (gall,),
        "1g": (1, gall),
    }[kind]


def batched_shape(kind: str, lall: int, kall: int, gall: int) -> tuple[int, ...]:
    """Shapes of the all-regions arrays of the reference harness (main.cpp:19-90)."""
    return {
        "kg": (lall, kall, gall),
        "qkg": (lall, NQ, kall, gall),
        "2g": (2, lall, gall),
        "g": (lall, gall),
        "1g": (lall, 1, gall),
    }[kind]


# ---------------------------------------------------------------- grid
def vertical_grid(kall: int, ztop: float = 40000.0) -> tuple[np.ndarray, np.ndarray]:
    """Full-level heights gz[kall] and interface heights gzh[kall] (kmin = 1, kmax = kall-2)."""
    if kall < 5:
        raise ValueError("kall must be >= 5")
    nlev = kall - 2
    gzh = np.zeros(kall)
    k = np.arange(1, kall)
    gzh[1:] = ztop * ((k - 1) / nlev) ** 1.5
    gzh[0] = -gzh[2]
    gz = np.zeros(kall)
    gz[1:kall - 1] = 0.5 * (gzh[1:kall - 1] + gzh[2:kall])
    gz[0] = -gz[1]
    gz[kall - 1] = 2.0 * gzh[kall - 1] - gz[kall - 2]
    return gz, gzh


def grid_factors(gz: np.ndarray, gzh: np.ndarray) -> dict[str, np.ndarray]:
    """Vertical metrics in the reference's GRD_Setup definitions (mod_debug.cpp:92-187)."""
    kall = gz.size
    kmin, kmax = 1, kall - 2
    dgz = np.zeros(kall)
    dgzh = np.zeros(kall)
    for k in range(kmin - 1, kmax + 1):
        dgz[k] = gzh[k + 1] - gzh[k]
    dgz[kmax + 1] = dgz[kmax]
    for k in range(kmin, kmax + 2):
        dgzh[k] = gz[k] - gz[k - 1]
    dgzh[kmin - 1] = dgzh[kmin]
    afact = np.zeros(kall)
    for k in range(kmin, kmax + 2):
        afact[k] = (gzh[k] - gz[k - 1]) / (gz[k] - gz[k - 1])
    afact[kmin - 1] = 1.0
    bfact = 1.0 - afact
    cfact = np.zeros(kall)
    for k in range(kmin, kmax + 1):
        cfact[k] = (gz[k] - gzh[k]) / (gzh[k + 1] - gzh[k])
    cfact[kmin - 1] = 1.0
    cfact[kmax + 1] = 0.0
    dfact = 1.0 - cfact
    return dict(dgz=dgz, dgzh=dgzh, rdgz=1.0 / dgz, rdgzh=1.0 / dgzh,
                afact=afact, bfact=bfact, cfact=cfact, dfact=dfact)


# ---------------------------------------------------------------- state
@dataclass(frozen=True)
class StateSpec:
    gall: int = 16900
    kall: int = 42
    lall: int = 1
    seed: int = 1001
    variant: str = "standard"      # standard | convective | cold
    dt: float = 60.0

    @property
    def cells(self) -> int:
        return self.gall * self.kall * self.lall


def _qsat_liq(tem: np.ndarray, rho: np.ndarray) -> np.ndarray:
    psat = PSAT0 * np.exp(LHV / RVAP * (1.0 / TEM00 - 1.0 / np.maximum(tem, 10.0)))
    return psat / (rho * RVAP * tem)


def make_region(rng: np.random.Generator, gall: int, kall: int, variant: str,
                gz: np.ndarray, gzh: np.ndarray) -> dict[str, np.ndarray]:
    """One region's mp_driver arguments, keyed by the reference argument names."""
    kmin, kmax = 1, kall - 2
    fac = grid_factors(gz, gzh)
    out: dict[str, np.ndarray] = {}

    lon = rng.uniform(0.0, 2.0 * np.pi, gall)
    lat = np.arcsin(rng.uniform(-1.0, 1.0, gall))
    ix, iy, iz = -np.sin(lon), np.cos(lon), np.zeros(gall)
    jx, jy, jz = -np.sin(lat) * np.cos(lon), -np.sin(lat) * np.sin(lon), np.cos(lat)

    z = np.repeat(gz[:, None], gall, axis=1)
    zh = np.repeat(gzh[:, None], gall, axis=1)
    gsgam2 = (1.0 + z / EARTH_RADIUS) ** 2
    gsgam2h = (1.0 + zh / EARTH_RADIUS) ** 2

    interior = slice(kmin, kmax + 1)
    zi = z[interior]
    t_sfc = 260.0 if variant == "cold" else 300.0
    tem = np.empty((kall, gall))
    tem[interior] = np.maximum(t_sfc - 6.5e-3 * zi, 210.0) + rng.normal(0.0, 1.0, zi.shape)

    # hydrostatic pressure from 1000 hPa at z = 0, trapezoidal temperature
    pre = np.empty((kall, gall))
    pre[kmin] = 1.0e5 * np.exp(-GRAV * gz[kmin] / (RDRY * tem[kmin]))
    for k in range(kmin + 1, kmax + 1):
        tbar = 0.5 * (tem[k] + tem[k - 1])
        pre[k] = pre[k - 1] * np.exp(-GRAV * (gz[k] - gz[k - 1]) / (RDRY * tbar))
    rho = np.empty((kall, gall))
    rho[interior] = pre[interior] / (RDRY * tem[interior])

    q = np.zeros((NQ, kall, gall))
    rh = rng.uniform(0.6, 1.05, zi.shape)
    ti = tem[interior]
    cloud = rng.random(zi.shape) < 0.30
    qcld = 1.0e-5 * np.exp(rng.normal(0.0, 1.0, zi.shape))
    q[I_QC][interior] = np.where(cloud & (ti > 273.0), qcld, 0.0)
    q[I_QI][interior] = np.where(cloud & (ti < 273.0), qcld, 0.0)
    for nq in (I_QR, I_QS, I_QG):
        on = rng.random(zi.shape) < 0.20
        q[nq][interior] = np.where(on, 1.0e-6 * np.exp(rng.normal(0.0, 1.0, zi.shape)), 0.0)

    if variant == "convective":
        conv = rng.random(gall) < 0.10
        low = (zi < 10000.0) & conv[None, :]
        rh = np.where(low, rng.uniform(1.0, 1.02, zi.shape), rh)
        q[I_QC][interior] = np.where(low & (ti > 273.0), np.maximum(q[I_QC][interior], 2.0e-4), q[I_QC][interior])
        qr_conv = np.minimum(5.0e-3, 1.0e-3 * np.exp(rng.normal(0.5, 0.6, zi.shape)))
        q[I_QR][interior] = np.where(low, qr_conv, q[I_QR][interior])

    q[I_QV][interior] = rh * _qsat_liq(ti, rho[interior])

    u = rng.normal(0.0, 10.0, (kall, gall))
    v = rng.normal(0.0, 10.0, (kall, gall))
    w = rng.normal(0.0, 1.0, (kall, gall))

    # halos are copies of the first and last layer
    for a in (tem, pre, rho, u, v):
        a[kmin - 1] = a[kmin]
        a[kmax + 1] = a[kmax]
    q[:, kmin - 1] = q[:, kmin]
    q[:, kmax + 1] = q[:, kmax]

    vx = u * ix + v * jx
    vy = u * iy + v * jy
    vz = u * iz + v * jz

    rhog = rho * gsgam2
    rhogq = rhog[None] * q
    q = rhogq / rhog[None]          # q is exactly rhogq / rhog, as the model keeps it
    qd = 1.0 - q[I_QC:].sum(axis=0)
    cv = qd * CVDRY + (q[I_QC:] * CVDRY).sum(axis=0)
    rhoge = rhog * cv * tem
    pre = rho * tem * (qd * RDRY + q[I_QV] * RVAP)

    # rhogw on half levels: w times the density interpolated to the level
    rhogh = np.zeros((kall, gall))
    for k in range(kmin, kmax + 2):
        c0 = fac["afact"][k] / gsgam2[k] * gsgam2h[k]
        c1 = fac["bfact"][k] / gsgam2[k - 1] * gsgam2h[k]
        rhogh[k] = c0 * rhog[k] + c1 * rhog[k - 1]
    rhogw = np.zeros((kall, gall))
    rhogw[kmin + 1:kmax + 1] = w[kmin + 1:kmax + 1] * rhogh[kmin + 1:kmax + 1]

    out.update(
        rhog=rhog, rhogvx=rhog * vx, rhogvy=rhog * vy, rhogvz=rhog * vz, rhogw=rhogw, rhoge=rhoge,
        rhogq=rhogq, vx=vx, vy=vy, vz=vz, w=w, unccn=np.zeros((kall, gall)),
        rho=rho, tem=tem, pre=pre, q=q,
        frhoge_af=np.zeros((kall, gall)), frhogqv_af=np.zeros((kall, gall)),
        frhoge_rad=np.zeros((kall, gall)), rhogqke=np.zeros((kall, gall)),
        gsgam2=gsgam2, gsgam2h=gsgam2h, gam2=gsgam2.copy(), gam2h=gsgam2h.copy(),
        ix=ix, iy=iy, iz=iz, jx=jx, jy=jy, jz=jz, z=z, zh=zh,
        CBMFX=np.zeros((kall, gall)),
    )
    return out


def region_rng(seed: int, l: int) -> np.random.Generator:
    """The random stream of region l: the seed's PCG64 stream for region 0,
    its l-th jump (2^127 draws ahead, an independent stream) for region l, so
    that any subset of regions can be generated on its own."""
    bitgen = np.random.PCG64(seed)
    return np.random.Generator(bitgen if l == 0 else bitgen.jumped(l))


def shard_regions(lall: int, rank: int, world: int) -> range:
    """The regions of one rank when `lall` regions are split over `world`
    ranks: contiguous blocks, the first lall % world ranks one region more.
    Regions are independent (the only cross-column coupling of the step, the
    departure-distance extrema, is per region), so every rank steps its block
    alone and no data moves between ranks."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside 0..{world - 1}")
    base, extra = divmod(lall, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def make_state(spec: StateSpec, out_fill: float = np.nan, regions=None) -> dict[str, np.ndarray]:
    """All-regions mp_driver arguments, arrays in the batched layout.

    Output-only arguments are filled with ``out_fill`` so that a test can
    check that every output element is written.  ``regions`` (default: all
    ``spec.lall``) selects the regions to generate, in that order; region l
    is the same array whichever subset it is generated in.
    """
    gz, gzh = vertical_grid(spec.kall)
    ls = range(spec.lall) if regions is None else list(regions)
    regions = [make_region(region_rng(spec.seed, l), spec.gall, spec.kall, spec.variant, gz, gzh) for l in ls]
    lall = len(regions)
    st: dict[str, np.ndarray] = {}
    for name, kind, intent in MP_DRIVER_ARGS:
        shp = batched_shape(kind, lall, spec.kall, spec.gall)
        if intent == "out":
            st[name] = np.full(shp, out_fill)
            continue
        if kind == "2g":
            st[name] = np.stack([r[name] for r in regions], axis=1)
        elif kind == "1g":
            st[name] = np.stack([r[name][None] for r in regions], axis=0)
        else:
            st[name] = np.stack([r[name] for r in regions], axis=0)
        st[name] = np.ascontiguousarray(st[name], dtype=np.float64)
    st["_gz"] = gz
    st["_gzh"] = gzh
    return st


def region_view(st: dict[str, np.ndarray], l: int) -> dict[str, np.ndarray]:
    """Contiguous copies of region ``l``'s arguments in the per-region layout."""
    out = {}
    for name, kind, _ in MP_DRIVER_ARGS:
        a = st[name]
        if kind == "2g":
            out[name] = np.ascontiguousarray(a[:, l])
        else:
            out[name] = np.ascontiguousarray(a[l])
    return out


def store_region(st: dict[str, np.ndarray], l: int, reg: dict[str, np.ndarray]) -> None:
    for name, kind, _ in MP_DRIVER_ARGS:
        if kind == "2g":
            st[name][:, l] = reg[name]
        else:
            st[name][l] = reg[name]


def regions_to_batched(regions: list[dict[str, np.ndarray]]) -> dict[str, np.ndarray]:
    """Stacks per-region argument sets (per-region layout, as region_view
    gives them) into the all-regions layout of mp_driver_batched."""
    out = {}
    for name, kind, _ in MP_DRIVER_ARGS:
        axis = 1 if kind == "2g" else 0
        out[name] = np.ascontiguousarray(np.stack([r[name] for r in regions], axis=axis), dtype=np.float64)
    return out
