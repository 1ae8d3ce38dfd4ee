"""Case descriptions: the ``&dns`` / ``&blocks`` namelist inputs of SNaC as Python data.

Mirrors the input of ``param.f90:68-277`` (``read_input``): global parameters
(``Case``) and one ``Block`` per entry of the ``&blocks`` namelist.  Boundary
condition arrays keep the reference's meaning and index order:
``cbcvel[comp][dir][side]`` is ``block_cbcvel(side,dir,comp,ib)``,
``cbcpre[dir][side]`` is ``block_cbcpre(side,dir,ib)``.  A friend link
(``'F'``) carries the 1-based id of the neighbouring block in the value array,
exactly as in the reference.

The factories below build the reference's lid-driven-cavity test
(tests/lid_driven_cavity/{dns,blocks}.nml) and the five benchmark cases:
a cubic lid-driven cavity, the triperiodic Taylor-Green vortex, the four-block
uneven turbulent channel, an L-shaped closed box and the differentially heated
cavity.  Initial conditions for cases the reference cannot generate natively
are produced here from documented formulas and seeds (the reference would
receive them through restart files, ``load.f90:84-153``).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

MAX_SCAL = 4


def bc6(s: str) -> List[List[str]]:
    """'FFDFDF' (the namelist order side-fastest, then direction) -> [dir][side]."""
    s = s.replace(",", "").replace(" ", "").replace("'", "")
    assert len(s) == 6
    return [[s[0], s[1]], [s[2], s[3]], [s[4], s[5]]]


def val6(v: Sequence[float]) -> List[List[float]]:
    assert len(v) == 6
    return [[float(v[0]), float(v[1])], [float(v[2]), float(v[3])], [float(v[4]), float(v[5])]]


@dataclasses.dataclass
class Block:
    ng: Sequence[int]
    lmin: Sequence[float]
    lmax: Sequence[float]
    cbcvel: List[List[List[str]]]
    bcvel: List[List[List[float]]]
    cbcpre: List[List[str]]
    bcpre: List[List[float]]
    gt: Sequence[int] = (0, 0, 0)
    gr: Sequence[float] = (0.0, 0.0, 0.0)
    cbcscal: Optional[List[List[List[str]]]] = None
    bcscal: Optional[List[List[List[float]]]] = None
    # optional axis grid files grid/grid_?_b_###.bin: rf, rc, drf, drc over lo..hi (4*ng doubles)
    grid_file: List[Optional[np.ndarray]] = dataclasses.field(default_factory=lambda: [None, None, None])
    # block_inflow_type(0:1,1:3): 0 none, 1 Poiseuille, 2 Kovasznay (param.f90:84)
    inflow_type: List[List[int]] = dataclasses.field(default_factory=lambda: [[0, 0], [0, 0], [0, 0]])

    @property
    def ncell(self) -> int:
        return int(self.ng[0]) * int(self.ng[1]) * int(self.ng[2])


@dataclasses.dataclass
class Case:
    name: str
    blocks: List[Block]
    visci: float = 1.0
    cfl: float = 0.95
    dtmax: float = 1.0e5
    dt_f: float = -1.0
    bforce: Sequence[float] = (0.0, 0.0, 0.0)
    gacc: Sequence[float] = (0.0, 0.0, 0.0)
    beta: float = 0.0
    nscal: int = 0
    alphai: Sequence[float] = ()
    ssource: Sequence[float] = ()
    scalf: Sequence[float] = ()
    is_sforced: Sequence[int] = ()
    icheck: int = 10
    fft_axis: int = 0          # 0: 3-D solve; 1..3 = FFT_AXIS build flag
    impdiff: int = 0
    boussinesq: int = 0
    tol: float = 1.0e-12       # relative residual of every Poisson/Helmholtz solve
    maxiter: int = 200

    @property
    def ncell(self) -> int:
        return sum(b.ncell for b in self.blocks)


# --------------------------------------------------------------------------- grids
def _gp_two_end(alpha: float, r0: float) -> float:
    """initgrid.f90:171-184 (gridpoint_cluster_two_end)."""
    if alpha != 0.0:
        return 0.5 * (1.0 + math.tanh((r0 - 0.5) * alpha) / math.tanh(alpha / 2.0))
    return r0


def global_axis_grid(n: int, lmin: float, lmax: float, alpha: float):
    """initgrid.f90:9-83 for one axis (two-end tanh clustering), indices 1..n.

    Returns (rf, rc, drf, drc) over 0..n+1 (index 0 and n+1 are the ghosts)."""
    rf = np.zeros(n + 2)
    drf = np.zeros(n + 2)
    drc = np.zeros(n + 2)
    rc = np.zeros(n + 2)
    for q in range(1, n + 1):
        r0 = (q - 1 + 1 - 0.0) / (1.0 * n)
        rf[q] = lmin + _gp_two_end(alpha, r0) * (lmax - lmin)
    rf[0] = lmin
    for q in range(1, n + 1):
        drf[q] = rf[q] - rf[q - 1]
    drf[0] = drf[1]
    drf[n + 1] = drf[n]
    for q in range(0, n + 1):
        drc[q] = 0.5 * (drf[q] + drf[q + 1])
    drc[n + 1] = drc[n]
    rc[0] = lmin - drc[0] / 2.0
    rf[0] = lmin
    for q in range(1, n + 2):
        rc[q] = rc[q - 1] + drc[q - 1]
        rf[q] = rf[q - 1] + drf[q]
    return rf, rc, drf, drc


def grid_file_slice(g, lo: int, hi: int) -> np.ndarray:
    """save_grid format (initgrid.f90:128-143): rf,rc,drf,drc over lo..hi (1-based)."""
    rf, rc, drf, drc = g
    return np.concatenate([rf[lo:hi + 1], rc[lo:hi + 1], drf[lo:hi + 1], drc[lo:hi + 1]]).astype(np.float64)


# --------------------------------------------------------------------------- cases
def _walls_block(ng, lmin, lmax, lid_u=0.0):
    """Closed single block, no-slip everywhere, optional lid u on the z+ face."""
    cbcvel = [bc6("DDDDDD")] * 3
    bcvel = [val6([0, 0, 0, 0, 0, lid_u]), val6([0] * 6), val6([0] * 6)]
    return Block(ng=ng, lmin=lmin, lmax=lmax, cbcvel=[list(map(list, c)) for c in cbcvel], bcvel=bcvel,
                 cbcpre=bc6("NNNNNN"), bcpre=val6([0] * 6))


def ldc_reference_test(fft_axis: int = 0, tol: float = 1e-12) -> Case:
    """tests/lid_driven_cavity/{dns,blocks}.nml: four 2x32x32 blocks, lid v=1 on z+ of blocks 3-4."""
    spec = [
        # lmin, lmax, cbcvel string, bcvel per component, cbcpre, bcpre
        ((0., 0., 0.), (0.3125, .5, .5), "FFDFDF", [(1, 1, 0, 2, 0, 3)] * 3, "FFNFNF", (1, 1, 0, 2, 0, 3)),
        ((0., .5, 0.), (0.3125, 1., .5), "FFFDDF", [(2, 2, 1, 0, 0, 4)] * 3, "FFFNNF", (2, 2, 1, 0, 0, 4)),
        ((0., 0., .5), (0.3125, .5, 1.), "FFDFFD", [(3, 3, 0, 4, 1, 0), (3, 3, 0, 4, 1, 1), (3, 3, 0, 4, 1, 0)],
         "FFNFFN", (3, 3, 0, 4, 1, 0)),
        ((0., .5, .5), (0.3125, 1., 1.), "FFFDFD", [(4, 4, 3, 0, 2, 0), (4, 4, 3, 0, 2, 1), (4, 4, 3, 0, 2, 0)],
         "FFFNFN", (4, 4, 3, 0, 2, 0)),
    ]
    blocks = []
    for lmin, lmax, cv, bv, cp, bp in spec:
        blocks.append(Block(ng=(2, 32, 32), lmin=lmin, lmax=lmax, cbcvel=[bc6(cv)] * 3,
                            bcvel=[val6(b) for b in bv], cbcpre=bc6(cp), bcpre=val6(bp)))
    return Case(name="ldc_reference_test", blocks=blocks, visci=1000.0, cfl=0.95, dtmax=1e5, dt_f=-1.0,
                icheck=10, fft_axis=fft_axis, tol=tol)


def lid_driven_cavity(n: int = 64, cfl: float = 0.5, tol: float = 1e-12) -> Case:
    """Config 1: single-block n^3 lid-driven cavity, Re=1000, 3-D multigrid."""
    b = _walls_block((n, n, n), (0., 0., 0.), (1., 1., 1.), lid_u=1.0)
    return Case(name=f"ldc{n}", blocks=[b], visci=1000.0, cfl=cfl, fft_axis=0, tol=tol)


def taylor_green(n: int = 128, tol: float = 1e-12) -> Case:
    """Config 2: triperiodic Taylor-Green vortex on [0,2pi]^3, FFT along z."""
    L = 2.0 * math.pi
    b = Block(ng=(n, n, n), lmin=(0., 0., 0.), lmax=(L, L, L), cbcvel=[bc6("FFFFFF")] * 3,
              bcvel=[val6([1] * 6)] * 3, cbcpre=bc6("FFFFFF"), bcpre=val6([1] * 6))
    return Case(name=f"tgv{n}", blocks=[b], visci=1600.0, cfl=0.95, fft_axis=3, tol=tol)


def channel_4block(nx=(96, 160), ny=(64, 80), nz: int = 128, stretch: float = 1.8,
                   lx: float = 4.0 * math.pi, ly: float = 2.0, lz: float = 4.0 * math.pi / 3.0,
                   tol: float = 1e-12) -> Case:
    """Config 3: turbulent channel in four uneven blocks (2 in x, 2 in y), FFT along z.

    Periodic x and z through friend links, no-slip walls in y with one global
    tanh two-end stretched wall-normal grid (initgrid.f90:171-184) split between
    the lower and upper block rows and passed as grid files."""
    nxt, nyt = nx[0] + nx[1], ny[0] + ny[1]
    gy = global_axis_grid(nyt, 0.0, ly, stretch)
    xs = [0.0, lx * nx[0] / nxt, lx]
    ysplit = float(gy[0][ny[0]])
    ys = [0.0, ysplit, ly]
    blocks = []
    # block ids: 1 (x0,y0) 2 (x1,y0) 3 (x0,y1) 4 (x1,y1)
    for jb in range(2):
        for ib in range(2):
            me = 1 + ib + 2 * jb
            xo = 1 + (1 - ib) + 2 * jb          # the other block of this row
            yo = 1 + ib + 2 * (1 - jb)          # the other block of this column
            ylo = ("D", 0.0) if jb == 0 else ("F", float(yo))
            yhi = ("F", float(yo)) if jb == 0 else ("D", 0.0)
            cv = ["F", "F", ylo[0], yhi[0], "F", "F"]
            vv = [xo, xo, ylo[1], yhi[1], me, me]
            cp = ["F", "F", "N" if ylo[0] == "D" else "F", "N" if yhi[0] == "D" else "F", "F", "F"]
            lo_y = 1 + (0 if jb == 0 else ny[0])
            hi_y = lo_y + ny[jb] - 1
            gf = [None, grid_file_slice(gy, lo_y, hi_y), None]
            blocks.append(Block(ng=(nx[ib], ny[jb], nz), lmin=(xs[ib], ys[jb], 0.0), lmax=(xs[ib + 1], ys[jb + 1], lz),
                                cbcvel=[bc6("".join(cv))] * 3, bcvel=[val6(vv)] * 3, cbcpre=bc6("".join(cp)),
                                bcpre=val6(vv), grid_file=gf))
    return Case(name="channel4", blocks=blocks, visci=180.0, cfl=0.95, bforce=(1.0, 0.0, 0.0), fft_axis=3, tol=tol)


def channel_4block_scalar(nx=(16, 32), ny=(8, 16), nz: int = 16, pr: float = 0.71, tol: float = 1e-12) -> Case:
    """The four-block channel with one passive scalar: T = 0 / 1 on the lower / upper wall, friend links
    elsewhere (as the velocity), bulk-forced to a mean of 0.5 (is_sforced, scal.f90:156-199)."""
    c = channel_4block(nx=nx, ny=ny, nz=nz, tol=tol)
    for b in c.blocks:
        cs = [list(f) for f in b.cbcpre]
        vs = [list(f) for f in b.bcpre]
        for side in range(2):
            if cs[1][side] == "N":  # a wall of the channel
                cs[1][side] = "D"
                vs[1][side] = 0.0 if side == 0 else 1.0
        b.cbcscal = [cs]
        b.bcscal = [vs]
    c.name = "channel4_scalar"
    c.nscal = 1
    c.alphai = (c.visci * pr,)
    c.ssource = (0.0,)
    c.scalf = (0.5,)
    c.is_sforced = (1,)
    return c


def dhc_reference_test() -> Case:
    """tests/differentially_heated_cavity/{dns,blocks}.nml: one 32x2x32 block, y periodic (FFT along y),
    no-slip walls in x and z, T = -0.5 / +0.5 on x- / x+, adiabatic z, Boussinesq buoyancy with
    gacc = (0, 0, -1), beta = 1, Ra = 1e8-like visci/alphai, fixed dt = 1e-3, explicit diffusion."""
    b = Block(ng=(32, 2, 32), lmin=(0.0, 0.0, 0.0), lmax=(1.0, 0.0625, 1.0),
              cbcvel=[bc6("DDFFDD")] * 3, bcvel=[val6([0, 0, 1, 1, 0, 0])] * 3,
              cbcpre=bc6("NNFFNN"), bcpre=val6([0, 0, 1, 1, 0, 0]),
              cbcscal=[bc6("DDFFNN")], bcscal=[val6([-0.5, 0.5, 1, 1, 0, 0])])
    return Case(name="dhc_reference_test", blocks=[b], visci=1186.78165819, cfl=0.95, dtmax=1e9, dt_f=1e-3,
                gacc=(0.0, 0.0, -1.0), beta=1.0, nscal=1, alphai=(842.614977318,), ssource=(0.0,), scalf=(0.0,),
                is_sforced=(0,), icheck=10, fft_axis=2, boussinesq=1, tol=1e-12)


def heated_cavity(n=(512, 512, 256), stretch: float = 1.5, ra: float = 1e8, pr: float = 0.71, impdiff: int = 1,
                  tol: float = 1e-12, dt_f: float = -1.0) -> Case:
    """Config 5: differentially heated cavity, one block on the unit box (n cells), tanh-stretched towards
    every wall (gt = 0, the two-end clustering of initgrid.f90, with gr = stretch), no-slip walls, T = +0.5 / -0.5
    on x- / x+ (hot / cold), adiabatic elsewhere, Boussinesq buoyancy with gacc = (0, 0, -1), beta = 1,
    visci = sqrt(Ra/Pr), alphai = sqrt(Ra Pr) (the convention of tests/differentially_heated_cavity),
    3-D pressure solve, implicit diffusion when impdiff (IMPDIFF)."""
    gr = max(stretch, 0.0)
    b = Block(ng=tuple(n), lmin=(0.0, 0.0, 0.0), lmax=(1.0, 1.0, 1.0), gt=(0, 0, 0), gr=(gr, gr, gr),
              cbcvel=[bc6("DDDDDD")] * 3, bcvel=[val6([0] * 6)] * 3, cbcpre=bc6("NNNNNN"), bcpre=val6([0] * 6),
              cbcscal=[bc6("DDNNNN")], bcscal=[val6([0.5, -0.5, 0, 0, 0, 0])])
    return Case(name=f"dhc{n[0]}x{n[1]}x{n[2]}", blocks=[b], visci=math.sqrt(ra / pr), cfl=0.95, dtmax=1e9,
                dt_f=dt_f, gacc=(0.0, 0.0, -1.0), beta=1.0, nscal=1, alphai=(math.sqrt(ra * pr),), ssource=(0.0,),
                scalf=(0.0,), is_sforced=(0,), icheck=10, fft_axis=0, impdiff=impdiff, boussinesq=1, tol=tol)


def dhc_initial_scalar(case: Case, xc_of_block):
    """initflow.f90:247-256 ('dhc'): T linear in x between the two wall values, on every cell incl. halo."""
    out = {}
    for ib, b in enumerate(case.blocks):
        xc = np.asarray(xc_of_block(ib))          # (nx+2) cell centres lo-1..hi+1
        lx = b.lmax[0] - b.lmin[0]
        t0, t1 = b.bcscal[0][0][0], b.bcscal[0][0][1]
        xx = xc / lx
        prof = (1.0 - xx) * t0 + xx * t1
        out[ib] = np.broadcast_to(prof[:, None, None], (b.ng[0] + 2, b.ng[1] + 2, b.ng[2] + 2)).copy()
    return out


def developing_duct(n=(32, 16, 16), inflow_type: int = 1, impdiff: int = 0, fft_axis: int = 0,
                    tol: float = 1e-12, dt_f: float = -1.0) -> Case:
    """The layout of examples/developing_duct: a square duct [0,1] x [0,1.5] x [0,1] with walls in y and z,
    an inflow on x- (inflow_type 1: the Poiseuille square-duct profile of init_inflow scaled to u = 1),
    zero-gradient velocity and p = 0 on x+, visci = 1000."""
    b = Block(ng=tuple(n), lmin=(0.0, 0.0, 0.0), lmax=(1.0, 1.5, 1.0),
              cbcvel=[bc6("DNDDDD"), bc6("NNDDDD"), bc6("NNDDDD")],
              bcvel=[val6([1, 0, 0, 0, 0, 0]), val6([0] * 6), val6([0] * 6)],
              cbcpre=bc6("NDNNNN"), bcpre=val6([0] * 6), inflow_type=[[inflow_type, 0], [0, 0], [0, 0]])
    return Case(name=f"duct{n[0]}x{n[1]}x{n[2]}", blocks=[b], visci=1000.0, cfl=0.95, dtmax=1e5, dt_f=dt_f,
                fft_axis=fft_axis, impdiff=impdiff, tol=tol)


def kovasznay(n=(40, 2, 16), visci: float = 40.0, impdiff: int = 0, tol: float = 1e-12, dt_f: float = -1.0) -> Case:
    """The layout of examples/__MULTI_BLOCK_GEOMETRY/kovasznay_flow: [-0.5,4.5] x [0,1/32] x [-0.5,0.5],
    periodic in y and z (self-friend faces), the Kovasznay inflow (inflow_type 2) on x-, zero-gradient
    velocity and p = 0 on x+; Re = visci (here 40, the classical case)."""
    b = Block(ng=tuple(n), lmin=(-0.5, 0.0, -0.5), lmax=(4.5, 0.03125, 0.5),
              cbcvel=[bc6("DNFFFF")] * 3,
              bcvel=[val6([1, 0, 1, 1, 1, 1]), val6([0, 0, 1, 1, 1, 1]), val6([0, 0, 1, 1, 1, 1])],
              cbcpre=bc6("NDFFFF"), bcpre=val6([0, 0, 1, 1, 1, 1]), inflow_type=[[2, 0], [0, 0], [0, 0]])
    return Case(name=f"kovasznay{n[0]}x{n[1]}x{n[2]}", blocks=[b], visci=visci, cfl=0.95, dtmax=1e5, dt_f=dt_f,
                fft_axis=0, impdiff=impdiff, tol=tol)


def l_shaped_box(n: int = 144, nz: int = 96, tol: float = 1e-12) -> Case:
    """Config 4: closed L-shaped box of three n x n x nz blocks (corner, +x leg, +y leg), lid u=1 on z+."""
    h = 1.0
    lz = h * nz / n
    # 1: corner [0,1]x[0,1]; 2: x-leg [1,2]x[0,1]; 3: y-leg [0,1]x[1,2]
    def blk(lmin, lmax, faces_vel, faces_pre, vals):
        return Block(ng=(n, n, nz), lmin=lmin, lmax=lmax,
                     cbcvel=[bc6(faces_vel)] * 3,
                     bcvel=[val6([vals[0], vals[1], vals[2], vals[3], vals[4], 1.0 if c == 0 else 0.0])
                            for c in range(3)], cbcpre=bc6(faces_pre), bcpre=val6(vals[:5] + [0.0]))
    b1 = blk((0, 0, 0), (h, h, lz), "DFDFDD", "NFNFNN", [0, 2, 0, 3, 0, 0])
    b2 = blk((h, 0, 0), (2 * h, h, lz), "FDDDDD", "FNNNNN", [1, 0, 0, 0, 0, 0])
    b3 = blk((0, h, 0), (h, 2 * h, lz), "DDFDDD", "NNFNNN", [0, 0, 1, 0, 0, 0])
    return Case(name="lbox", blocks=[b1, b2, b3], visci=2000.0, cfl=0.95, fft_axis=0, tol=tol)


# --------------------------------------------------------------------------- initial conditions
def splitmix64_uniform(seed: int, n: int) -> np.ndarray:
    """Uniform [0,1) doubles from the splitmix64 sequence (53-bit mantissa), reproducible everywhere."""
    mask = (1 << 64) - 1
    out = np.empty(n, dtype=np.float64)
    x = seed & mask
    for q in range(n):
        x = (x + 0x9E3779B97F4A7C15) & mask
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z = z ^ (z >> 31)
        out[q] = (z >> 11) * (1.0 / (1 << 53))
    return out


def channel_bulk_velocity(case: Case) -> float:
    """Bulk velocity of the turbulent-channel estimate of initflow.f90 ('pdc', is_wallturb):
    u_tau = sqrt(bforce*h), Re_b = (Re_tau/0.09)**(1/0.88), U_b = Re_b*visc/(2h), h = half height = 1."""
    lref = 1.0
    uref = math.sqrt(case.bforce[0] * lref)
    visc = 1.0 / case.visci
    retau = uref * lref / visc
    reb = (retau / 0.09) ** (1.0 / 0.88)
    return reb * visc / (2.0 * lref)


def channel_initial_condition(case: Case, yc_of_block, seed: int = 0x5EED, amp: float = 0.1):
    """Laminar Poiseuille profile in y scaled to U_b plus uniform noise in [-amp, amp]*U_b on u, v, w.

    yc_of_block(ib) returns the (ng+2) cell-centre y coordinates of block ib.  Noise values are drawn
    from one splitmix64 stream, block by block, component by component, Fortran order of the interior.
    Returns {ib: (u, v, w)} halo'd arrays (ghosts zero)."""
    ub = channel_bulk_velocity(case)
    out = {}
    offset = 0
    for ib, b in enumerate(case.blocks):
        n = [int(x) for x in b.ng]
        ncell = n[0] * n[1] * n[2]
        yc = yc_of_block(ib)[1:-1]
        prof = 1.5 * ub * yc * (2.0 - yc)
        comps = []
        for c in range(3):
            r = splitmix64_uniform_fast(seed + offset, ncell).reshape(n, order="F")
            offset += ncell
            f = np.zeros([x + 2 for x in n], order="F")
            f[1:-1, 1:-1, 1:-1] = 2.0 * (r - 0.5) * amp * ub
            if c == 0:
                f[1:-1, 1:-1, 1:-1] += prof[None, :, None]
            comps.append(f)
        out[ib] = tuple(comps)
    return out


def tgv_initial_condition(case: Case, grid):
    """Taylor-Green vortex on the MAC grid: u = sin x cos y cos z at the x faces, v = -cos x sin y cos z at the
    y faces, w = 0, and the analytic pressure p = (cos 2x + cos 2y)(cos 2z + 2)/16 at the cell centres.

    grid(ib, axis, which) returns the (ng+2) coordinates of block ib (which = G_XC centres, G_XF faces).
    Returns {ib: (u, v, w, p)} halo'd arrays, ghosts included."""
    from .capi import G_XC, G_XF
    out = {}
    for ib, _ in enumerate(case.blocks):
        xc, yc, zc = (grid(ib, a, G_XC) for a in range(3))
        xf, yf = grid(ib, 0, G_XF), grid(ib, 1, G_XF)
        u = np.asfortranarray(np.sin(xf)[:, None, None] * np.cos(yc)[None, :, None] * np.cos(zc)[None, None, :])
        v = np.asfortranarray(-np.cos(xc)[:, None, None] * np.sin(yf)[None, :, None] * np.cos(zc)[None, None, :])
        w = np.zeros_like(u, order="F")
        p = np.asfortranarray((np.cos(2 * xc)[:, None, None] + np.cos(2 * yc)[None, :, None])
                              * (np.cos(2 * zc)[None, None, :] + 2.0) / 16.0)
        out[ib] = (u, v, w, p)
    return out


def splitmix64_uniform_fast(seed: int, n: int) -> np.ndarray:
    """Vectorised splitmix64 (identical output to splitmix64_uniform)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        x = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
