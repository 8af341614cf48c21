"""Seeded synthetic CSEM models and acquisitions in the reference's file formats.

The reference driver reads (emf_init_free.c:77-150, acq_init_free.c:38-81):
  * fx1, fx2, fx3: float32 node coordinates, nx+1 / ny+1 / nz+1 values (the cell
    counts are inferred from the file sizes);
  * frho11, frho22, frho33: float32 cell resistivities, nx*ny*nz values, x fastest,
    then y, then z;
  * sources.txt / receivers.txt: one header line, then rows of
    "x1 x2 x3 azimuth dip index" (at most 5000 rows, acq_init_free.c:17).

The builders below produce the workloads the GPU solver is measured on:
  layered_120     100x100x100 cells of 100 m, x,y in [-5,5] km, z in [0,10] km,
                  0.3 ohm-m water above 1000 m, 1 ohm-m below, 100 ohm-m at 2000-2100 m;
                  one Ex dipole at (0,0,950); 101 seafloor receivers (y=0, z=1000).
  vti_block_120   the same grid, rho33 = 2*rho11, plus a 50 ohm-m 2x2x0.1 km block
                  centred at (0,0,2050).
  marlim_like     180x120x120 cells (200 m in x, 100 m in y,z), seafloor at 1500 m,
                  30 seeded layers of 100 m (rho11=rho22 log-uniform in [0.5,5],
                  rho33 = 1.5*rho11), 4 seeded ellipsoidal 20-100 ohm-m resistors;
                  16 Ex sources every 1 km on y=0, 50 m above the seafloor;
                  181 seafloor receivers every 200 m on y=0.
  random_small    small random grids for operator parity tests.
Every builder is deterministic for a given seed (numpy default_rng).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Model:
    x1: np.ndarray  # float32 node coordinates, nx+1
    x2: np.ndarray
    x3: np.ndarray
    rho11: np.ndarray  # float32 [nz][ny][nx]
    rho22: np.ndarray
    rho33: np.ndarray
    name: str = "model"

    @property
    def shape(self):
        return (len(self.x1) - 1, len(self.x2) - 1, len(self.x3) - 1)


@dataclass
class Acquisition:
    src: np.ndarray  # float32 [nsrc][5]: x1 x2 x3 azimuth dip
    rec: np.ndarray  # float32 [nrec][5]


@dataclass
class Config:
    """One workload: a model, an acquisition and the reference driver's flags."""
    model: Model
    acq: Acquisition
    params: dict = field(default_factory=dict)
    name: str = "config"

    def args(self, workdir: str, isrc: int = 0) -> list[str]:
        """key=value argument list for the reference-style driver in `workdir`."""
        a = ["csem"]
        for k, v in self.params.items():
            a.append(f"{k}={v}")
        a += [f"fx1={workdir}/fx1", f"fx2={workdir}/fx2", f"fx3={workdir}/fx3",
              f"frho11={workdir}/frho11", f"frho22={workdir}/frho22",
              f"frho33={workdir}/frho33",
              f"fsrc={workdir}/sources_{isrc:04d}.txt" if isrc else f"fsrc={workdir}/sources.txt",
              f"frec={workdir}/receivers.txt"]
        return a


def write_model(model: Model, d: str) -> None:
    os.makedirs(d, exist_ok=True)
    for nm in ("x1", "x2", "x3"):
        np.asarray(getattr(model, nm), dtype=np.float32).tofile(os.path.join(d, "f" + nm))
    for nm in ("rho11", "rho22", "rho33"):
        np.ascontiguousarray(getattr(model, nm), dtype=np.float32).tofile(os.path.join(d, "f" + nm))


def _write_rows(path: str, rows: np.ndarray, tag: str) -> None:
    with open(path, "w") as f:
        f.write(f"          x1          x2          x3     azimuth         dip         {tag}\n")
        for i, r in enumerate(rows):
            f.write(f"{r[0]:.6f} {r[1]:.6f} {r[2]:.6f} {r[3]:.6f} {r[4]:.6f} {i + 1}\n")


def write_acquisition(acq: Acquisition, d: str) -> None:
    """sources.txt holds every source (the reference solves only its first row);
    sources_NNNN.txt (1-based) hold one source each for per-source drivers."""
    os.makedirs(d, exist_ok=True)
    _write_rows(os.path.join(d, "sources.txt"), acq.src, "iTx")
    for i in range(len(acq.src)):
        _write_rows(os.path.join(d, f"sources_{i + 1:04d}.txt"), acq.src[i:i + 1], "iTx")
    _write_rows(os.path.join(d, "receivers.txt"), acq.rec, "iRx")


def write_config(cfg: Config, d: str) -> None:
    write_model(cfg.model, d)
    write_acquisition(cfg.acq, d)


def _centres(x):
    x = np.asarray(x, dtype=np.float64)
    return 0.5 * (x[:-1] + x[1:])


def layered_120(freqs=(0.25, 0.75, 1.25)) -> Config:
    x1 = np.arange(-5000, 5001, 100, dtype=np.float32)
    x2 = x1.copy()
    x3 = np.arange(0, 10001, 100, dtype=np.float32)
    zc = _centres(x3)
    rho_z = np.where(zc < 1000, 0.3, 1.0)
    rho_z = np.where((zc >= 2000) & (zc < 2100), 100.0, rho_z)
    rho = np.broadcast_to(rho_z[:, None, None], (100, 100, 100)).astype(np.float32)
    model = Model(x1, x2, x3, rho.copy(), rho.copy(), rho.copy(), name="layered_120")
    src = np.array([[0, 0, 950, 0, 0]], dtype=np.float32)
    rx = np.arange(-5000, 5001, 100, dtype=np.float32)
    rec = np.stack([rx, np.zeros_like(rx), np.full_like(rx, 1000), np.zeros_like(rx),
                    np.zeros_like(rx)], axis=1).astype(np.float32)
    params = dict(airbc=1, nb=10, lextend="40e3", preco=1, algopt=1, tol="1e-8", niter=1000,
                  fvm=0, chsrc="Ex", chrec="Ex,Ey,Ez",
                  freqs=",".join(str(f) for f in freqs))
    return Config(model, Acquisition(src, rec), params, name="layered_120")


def vti_block_120(freqs=(0.25, 0.75, 1.25)) -> Config:
    cfg = layered_120(freqs)
    m = cfg.model
    xc, yc, zc = _centres(m.x1), _centres(m.x2), _centres(m.x3)
    blk = ((np.abs(xc)[None, None, :] <= 1000) & (np.abs(yc)[None, :, None] <= 1000)
           & ((zc >= 2000) & (zc < 2100))[:, None, None])
    r11 = np.where(blk, 50.0, m.rho11).astype(np.float32)
    m.rho11 = r11
    m.rho22 = r11.copy()
    m.rho33 = (2.0 * r11).astype(np.float32)
    m.name = "vti_block_120"
    cfg.name = "vti_block_120"
    return cfg


def marlim_like(seed: int = 0, freqs=(0.125, 0.25, 0.5, 0.75, 1.0, 1.25), nsrc: int = 16) -> Config:
    rng = np.random.default_rng(seed)
    x1 = np.arange(-18000, 18001, 200, dtype=np.float32)   # 180 cells
    x2 = np.arange(-6000, 6001, 100, dtype=np.float32)     # 120 cells
    x3 = np.arange(0, 12001, 100, dtype=np.float32)        # 120 cells
    xc, yc, zc = _centres(x1), _centres(x2), _centres(x3)
    nz, ny, nx = len(zc), len(yc), len(xc)
    seafloor = 1500.0
    rho11 = np.full((nz, ny, nx), 0.3)
    layer_rho = np.exp(rng.uniform(np.log(0.5), np.log(5.0), size=30))
    for L in range(30):
        top, bot = seafloor + 100 * L, seafloor + 100 * (L + 1)
        sel = (zc >= top) & (zc < bot)
        rho11[sel] = layer_rho[L]
    below = zc >= seafloor + 3000
    rho11[below] = layer_rho[-1]
    rho33 = np.where(zc[:, None, None] >= seafloor, 1.5 * rho11, rho11)
    Z, Y, X = np.meshgrid(zc, yc, xc, indexing="ij")
    for _ in range(4):
        r = rng.uniform(20, 100)
        ax, ay, az = rng.uniform(500, 3000), rng.uniform(500, 3000), rng.uniform(50, 200)
        cx = rng.uniform(-12000, 12000)
        cy = rng.uniform(-3000, 3000)
        cz = rng.uniform(seafloor + 400, seafloor + 2600)
        inside = ((X - cx) / ax) ** 2 + ((Y - cy) / ay) ** 2 + ((Z - cz) / az) ** 2 <= 1.0
        rho11 = np.where(inside, r, rho11)
        rho33 = np.where(inside, r, rho33)
    model = Model(x1, x2, x3, rho11.astype(np.float32), rho11.astype(np.float32),
                  rho33.astype(np.float32), name="marlim_like")
    sx = -7500.0 + 1000.0 * np.arange(nsrc)
    src = np.stack([sx, np.zeros(nsrc), np.full(nsrc, seafloor - 50.0), np.zeros(nsrc),
                    np.zeros(nsrc)], axis=1).astype(np.float32)
    rx = np.arange(-18000, 18001, 200, dtype=np.float64)
    rec = np.stack([rx, np.zeros_like(rx), np.full_like(rx, seafloor), np.zeros_like(rx),
                    np.zeros_like(rx)], axis=1).astype(np.float32)
    params = dict(airbc=1, nb=10, lextend="120e3", preco=1, algopt=1, tol="1e-8", niter=1000,
                  fvm=0, chsrc="Ex", chrec="Ex,Ey,Ez",
                  freqs=",".join(str(f) for f in freqs))
    return Config(model, Acquisition(src, rec), params, name="marlim_like")


def large_420(seed: int = 2, freqs=(0.125, 0.25, 0.5, 0.75, 1.0, 1.25), nsrc: int = 32) -> Config:
    """Large memory-bound batch: 400x400x200 core cells of 50 m padded by nb=10 to
    420x420x220 (about 116M complex edge unknowns per system), a seeded layered
    anisotropic model built as marlim_like (seafloor 1500 m, 30 layers of 100 m,
    rho33 = 1.5 rho11) with 8 seeded resistors; 32 Ex sources along y=0, 6 frequencies:
    192 systems, solved in waves that fit device memory."""
    rng = np.random.default_rng(seed)
    x1 = np.arange(-10000, 10001, 50, dtype=np.float32)
    x2 = x1.copy()
    x3 = np.arange(0, 10001, 50, dtype=np.float32)
    xc, yc, zc = _centres(x1), _centres(x2), _centres(x3)
    nz, ny, nx = len(zc), len(yc), len(xc)
    seafloor = 1500.0
    layer_rho = np.exp(rng.uniform(np.log(0.5), np.log(5.0), size=30))
    rz = np.full(nz, 0.3)
    for L in range(30):
        rz[(zc >= seafloor + 100 * L) & (zc < seafloor + 100 * (L + 1))] = layer_rho[L]
    rz[zc >= seafloor + 3000] = layer_rho[-1]
    rho11 = np.broadcast_to(rz[:, None, None], (nz, ny, nx)).astype(np.float32).copy()
    rho33 = np.broadcast_to(np.where(zc >= seafloor, 1.5 * rz, rz)[:, None, None], (nz, ny, nx)).astype(np.float32).copy()
    for _ in range(8):
        r = rng.uniform(20, 100)
        ax, ay, az = rng.uniform(500, 3000), rng.uniform(500, 3000), rng.uniform(50, 200)
        cx, cy = rng.uniform(-7000, 7000), rng.uniform(-7000, 7000)
        cz = rng.uniform(seafloor + 400, seafloor + 2600)
        kz = np.nonzero(np.abs(zc - cz) <= az)[0]
        jy = np.nonzero(np.abs(yc - cy) <= ay)[0]
        ix = np.nonzero(np.abs(xc - cx) <= ax)[0]
        if not (len(kz) and len(jy) and len(ix)):
            continue
        Z, Y, X = np.meshgrid(zc[kz], yc[jy], xc[ix], indexing="ij")
        inside = ((X - cx) / ax) ** 2 + ((Y - cy) / ay) ** 2 + ((Z - cz) / az) ** 2 <= 1.0
        sub = np.ix_(kz, jy, ix)
        rho11[sub] = np.where(inside, r, rho11[sub])
        rho33[sub] = np.where(inside, r, rho33[sub])
    model = Model(x1, x2, x3, rho11, rho11.copy(), rho33, name="large_420")
    sx = -7750.0 + 500.0 * np.arange(nsrc)
    src = np.stack([sx, np.zeros(nsrc), np.full(nsrc, seafloor - 50.0), np.zeros(nsrc),
                    np.zeros(nsrc)], axis=1).astype(np.float32)
    rx = np.arange(-9800, 9801, 200, dtype=np.float64)
    rec = np.stack([rx, np.zeros_like(rx), np.full_like(rx, seafloor), np.zeros_like(rx),
                    np.zeros_like(rx)], axis=1).astype(np.float32)
    params = dict(airbc=1, nb=10, lextend="40e3", preco=1, algopt=1, tol="1e-8", niter=1000,
                  fvm=0, chsrc="Ex", chrec="Ex,Ey,Ez",
                  freqs=",".join(str(f) for f in freqs))
    return Config(model, Acquisition(src, rec), params, name="large_420")


def _layered_cells(x3, surfaces, rho_layers):
    """Cell resistivities of layers separated by depth surfaces ([ny][nx] each, top to
    bottom), averaged over each cell's vertical extent: conductivity arithmetically for
    the horizontal components and resistivity arithmetically for the vertical one (the
    volume-fraction averaging of the reference's bathymetry example,
    bathymetry/main.c:25-104). Returns rho_h, rho_v as float32 [nz][ny][nx]."""
    ztop = np.asarray(x3[:-1], np.float64)[:, None, None]
    zbot = np.asarray(x3[1:], np.float64)[:, None, None]
    dz = zbot - ztop
    cuts = [None] + [np.asarray(sf, np.float64)[None] for sf in surfaces] + [None]
    sig = np.zeros((len(ztop),) + np.shape(surfaces[0]))
    rv = np.zeros_like(sig)
    for L, rho in enumerate(rho_layers):
        lo = ztop if cuts[L] is None else np.maximum(ztop, cuts[L])
        hi = zbot if cuts[L + 1] is None else np.minimum(zbot, cuts[L + 1])
        frac = np.clip(hi - lo, 0.0, None) / dz
        sig += frac / rho
        rv += frac * rho
    return (1.0 / sig).astype(np.float32), rv.astype(np.float32)


def bathymetry_125(seed: int = 1, freqs=(0.25, 0.75, 1.25), nsrc: int = 8) -> Config:
    """125x125x100 cells of 100 m; seafloor at 1000 m plus 3 seeded Gaussian hills
    (amplitude 200-500 m, sigma 1-3 km); 0.3 ohm-m water above it, 1 ohm-m below, and a
    30 ohm-m layer 100 m thick following the topography 800 m beneath it; partial cells
    averaged by volume fraction. Ex sources every 1 km on y=0, 50 m above the local
    seafloor; receivers on the seafloor along y=0 every 200 m."""
    rng = np.random.default_rng(seed)
    x1 = np.arange(-6250, 6251, 100, dtype=np.float32)
    x2 = x1.copy()
    x3 = np.arange(0, 10001, 100, dtype=np.float32)
    xc, yc = _centres(x1), _centres(x2)
    X, Y = np.meshgrid(xc, yc)
    hills = [(rng.uniform(200, 500), rng.uniform(1000, 3000), rng.uniform(-4000, 4000), rng.uniform(-4000, 4000))
             for _ in range(3)]

    def seafloor(x, y):
        return 1000.0 + sum(a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sg * sg)) for a, sg, cx, cy in hills)

    sf = seafloor(X, Y)
    rh, rv = _layered_cells(x3, [sf, sf + 800.0, sf + 900.0], [0.3, 1.0, 30.0, 1.0])
    model = Model(x1, x2, x3, rh, rh.copy(), rv, name="bathymetry_125")
    sx = -3500.0 + 1000.0 * np.arange(nsrc)
    src = np.stack([sx, np.zeros(nsrc), seafloor(sx, 0.0) - 50.0, np.zeros(nsrc), np.zeros(nsrc)],
                   axis=1).astype(np.float32)
    rx = np.arange(-6000, 6001, 200, dtype=np.float64)
    rec = np.stack([rx, np.zeros_like(rx), seafloor(rx, 0.0), np.zeros_like(rx), np.zeros_like(rx)],
                   axis=1).astype(np.float32)
    params = dict(airbc=1, nb=10, lextend="40e3", preco=3, algopt=2, nrestart=10, tol="1e-8", niter=1000,
                  fvm=0, chsrc="Ex", chrec="Ex,Ey,Ez", freqs=",".join(str(f) for f in freqs))
    return Config(model, Acquisition(src, rec), params, name="bathymetry_125")


def layered_64(freqs=(0.25, 0.75, 1.25)) -> Config:
    """64^3 cells of 100 m: 0.3 ohm-m water above 1000 m, 1 ohm-m below, 100 ohm-m at
    2000-2100 m; one Ex dipole at (0, 0, 950) and seafloor receivers along y=0."""
    x1 = np.arange(-3200, 3201, 100, dtype=np.float32)
    x2 = x1.copy()
    x3 = np.arange(0, 6401, 100, dtype=np.float32)
    zc = _centres(x3)
    rz = np.where(zc < 1000, 0.3, 1.0)
    rz = np.where((zc >= 2000) & (zc < 2100), 100.0, rz)
    rho = np.broadcast_to(rz[:, None, None], (64, 64, 64)).astype(np.float32)
    model = Model(x1, x2, x3, rho.copy(), rho.copy(), rho.copy(), name="layered_64")
    src = np.array([[0, 0, 950, 0, 0]], dtype=np.float32)
    rx = np.arange(-3000, 3001, 100, dtype=np.float64)
    rec = np.stack([rx, np.zeros_like(rx), np.full_like(rx, 1000.0), np.zeros_like(rx), np.zeros_like(rx)],
                   axis=1).astype(np.float32)
    params = dict(airbc=1, nb=10, lextend="40e3", preco=3, algopt=2, nrestart=10, tol="1e-8", niter=1000,
                  fvm=0, chsrc="Ex", chrec="Ex,Ey,Ez", freqs=",".join(str(f) for f in freqs))
    return Config(model, Acquisition(src, rec), params, name="layered_64")


def random_small(seed: int, nx=12, ny=10, nz=9, airbc=0, nb=3, aniso=True, stretch=True,
                 freqs=(0.5, 1.0), **extra) -> Config:
    """Small random model: random (optionally stretched) node spacings, random
    log-uniform resistivities with a 0.3 ohm-m water layer on top, one Ex source
    and a few receivers inside the core. Used for per-operator parity."""
    rng = np.random.default_rng(seed)

    def axis(n, d0):
        if stretch:
            d = d0 * rng.uniform(0.7, 1.5, size=n)
        else:
            d = np.full(n, d0)
        x = np.concatenate([[0.0], np.cumsum(d)])
        return (x - x[-1] / 2).astype(np.float32)

    x1 = axis(nx, 100.0)
    x2 = axis(ny, 100.0)
    x3 = axis(nz, 100.0)
    x3 = (x3 - x3[0]).astype(np.float32)
    zc = _centres(x3)
    r = np.exp(rng.uniform(np.log(0.5), np.log(20.0), size=(nz, ny, nx)))
    r[zc < x3[2], :, :] = 0.3
    r11 = r.astype(np.float32)
    r22 = (r * (rng.uniform(0.8, 1.25, size=r.shape) if aniso else 1)).astype(np.float32)
    r33 = (r * (rng.uniform(1.0, 3.0, size=r.shape) if aniso else 1)).astype(np.float32)
    r22[zc < x3[2], :, :] = 0.3
    r33[zc < x3[2], :, :] = 0.3
    model = Model(x1, x2, x3, r11, r22, r33, name=f"random_small_{seed}")
    c1 = _centres(x1)
    c2 = _centres(x2)
    src = np.array([[0.37 * c1[nx // 2] + 11.0, 0.41 * c2[ny // 2] + 7.0, float(x3[2]) - 23.0, 0, 0]],
                   dtype=np.float32)
    nrec = 5
    rx = np.linspace(x1[1], x1[-2], nrec)
    rec = np.stack([rx, np.full(nrec, 0.5 * (x2[1] + x2[2])), np.full(nrec, float(x3[2])),
                    np.zeros(nrec), np.zeros(nrec)], axis=1).astype(np.float32)
    params = dict(airbc=airbc, nb=nb, preco=1, algopt=1, tol="1e-8", niter=50, fvm=0,
                  chsrc="Ex", chrec="Ex,Ey,Ez", freqs=",".join(str(f) for f in freqs),
                  lextend="3000")
    params.update(extra)
    return Config(model, Acquisition(src, rec), params, name=model.name)


WORKLOADS = {"marlim_like_96": lambda: marlim_like(seed=0), "layered_120": layered_120,
             "vti_block_120": vti_block_120, "large_420_192": lambda: large_420(seed=2),
             "bathymetry_125": bathymetry_125, "layered_64": layered_64}


def workload(name: str) -> Config:
    """A named workload (marlim_like_96, layered_120, vti_block_120, large_420_192,
    bathymetry_125, layered_64)."""
    if name not in WORKLOADS:
        raise ValueError(f"unknown workload {name}; known: {', '.join(WORKLOADS)}")
    return WORKLOADS[name]()


def build_grid(cfg: Config, d: str):
    """Write `cfg` into directory d and run the product's host set-up on it (read,
    extend with the config's nb/lextend, airwave tables when airbc=1)."""
    from .api import Grid
    write_config(cfg, d)
    p = cfg.params
    G = Grid.from_files(*[os.path.join(d, n) for n in ("fx1", "fx2", "fx3", "frho11", "frho22", "frho33")])
    G.extend(int(p.get("nb", 15)), float(p.get("lextend", -1)), float(p.get("rho_air", 1e6)), int(p.get("istretch", 1)))
    if int(p.get("airbc", 0)):
        G.airbc(int(p.get("n1fft", 1024)), int(p.get("n2fft", 1024)))
    return G
