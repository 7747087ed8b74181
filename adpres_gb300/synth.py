"""Seeded synthetic cores, written as ADPRES input decks.

There is no public dataset for this path: the workloads are cores of the
shapes the solver is measured on, generated from numpy seeds and emitted in
the reference's own card format, so the same text feeds both the CUDA path
and the CPU oracle.

  quarter_core_2d  9x9 assemblies of 20 cm, 2x2 nodes each, one axial layer
                   (two identical 10 cm planes between reflective planes),
                   2 groups, SANM.
  full_core_3d     17x17 assemblies, 2x2 nodes each, 20 fuel layers of 20 cm
                   plus one reflector layer top and bottom, corner assemblies
                   reflector, 3 fuel types, rodded top 40% in 8 assemblies.
  core_4g          17x17 assemblies with 4x4 nodes, 80 planes of 5 cm,
                   4 groups with down-scatter only.
  batch_member     a 2-group core with a drawn radial grid (20..68 nodes),
                   axial size (10..40 nodes) and a cylindrical outline (fuel
                   inside, one reflector ring), cross sections perturbed by
                   1% lognormal factors per material value.
  boron_search_3d  the full-core geometry in mode BCSEARCH with boron, fuel
                   and moderator temperature, coolant density and two
                   control-rod banks as feedback cards.
  rod_ejection_3d  the same core in mode RODEJECT: one bank ejected in 0.05 s.
  small_core       a small ragged core with optional ADFs, any boundary
                   conditions and 1-4 groups (parity tests).

Fission cross sections for the power edit are nu*Sigma_f / 2.43.
"""
from __future__ import annotations

import numpy as np

NU = 2.43

# Reflector of the 2-group configurations: D1 1.30, D2 0.27 cm; Sa 0.001 / 0.020; S12 0.030.
REFL2 = dict(D=(1.30, 0.27), sa=(0.001, 0.020), nuf=(0.0, 0.0), s12=0.030)
FUEL_RANGES = dict(D1=(1.40, 1.50), D2=(0.38, 0.42), sa1=(0.009, 0.011), sa2=(0.080, 0.100),
                   nuf1=(0.005, 0.007), nuf2=(0.12, 0.14), s12=(0.016, 0.020))


def _fmt(v):
    return repr(float(v))


def _mat2(D, sa, nuf, s12, chi=(1.0, 0.0)):
    """(ng=2) material rows: sigtr siga nuf sigf chi sigs(g->1) sigs(g->2)."""
    sigtr = [1.0 / (3.0 * d) for d in D]
    sigf = [x / NU for x in nuf]
    rows = [[sigtr[0], sa[0], nuf[0], sigf[0], chi[0], 0.0, s12],
            [sigtr[1], sa[1], nuf[1], sigf[1], chi[1], 0.0, 0.0]]
    return rows


def _fuel2(rng):
    r = FUEL_RANGES
    u = lambda k: rng.uniform(*r[k])
    return dict(D=(u("D1"), u("D2")), sa=[u("sa1"), u("sa2")], nuf=(u("nuf1"), u("nuf2")), s12=u("s12"))


def _deck(name, ng, mats, nx, ny, nz, xsize, xdiv, ysize, ydiv, zsize, zdiv, planars, zpln, bc,
          kern="SANM", iter_=None, adf=None, mode="FORWARD"):
    L = ["! synthetic core generated by adpres_gb300.synth", "%MODE", mode, "%CASE", name, "SYNTHETIC", "%KERN", kern,
         "%XSEC", f"{ng} {len(mats)}"]
    for rows in mats:
        for row in rows:
            L.append(" ".join(_fmt(v) for v in row))
    L += ["%GEOM", f"{nx} {ny} {nz}",
          " ".join(_fmt(v) for v in xsize), " ".join(str(int(v)) for v in xdiv),
          " ".join(_fmt(v) for v in ysize), " ".join(str(int(v)) for v in ydiv),
          " ".join(_fmt(v) for v in zsize), " ".join(str(int(v)) for v in zdiv),
          str(len(planars)), " ".join(str(int(v)) for v in zpln)]
    for pl in planars:                      # pl[i][j] with j = 0 south; written north row first
        for j in range(ny - 1, -1, -1):
            L.append(" ".join(str(int(pl[i][j])) for i in range(nx)))
    L.append(" ".join(str(int(b)) for b in bc))
    if iter_ is not None:
        L += ["%ITER", " ".join(str(v) for v in iter_)]
    if adf is not None:
        L.append("%ADF")
        for rows in adf:
            for row in rows:
                L.append(" ".join(_fmt(v) for v in row))
        L += ["0"]
    return "\n".join(L) + "\n"


def _nupd(nxx, nyy, nzz):
    return int(np.ceil(np.float32(nxx + nyy + nzz) / np.float32(2.5)))


def quarter_core_2d(seed=0, nout=2000):
    """Quarter core, 9x9 assemblies, reflective west/north, zero incoming current east/south."""
    rng = np.random.default_rng(seed)
    fa, fb = _fuel2(rng), _fuel2(rng)
    mats = [_mat2(**REFL2), _mat2(**fa), _mat2(**fb)]
    nx = ny = 9
    pl = np.zeros((nx, ny), dtype=int)
    for i in range(nx):
        for j in range(ny):
            outer = (i == nx - 1) or (j == 0)     # east column and south row
            pl[i, j] = 1 if outer else int(rng.integers(2, 4))
    nxx, nyy, nzz = 18, 18, 2
    it = [nout, 2, "1.0e-5", "1.0e-5", 5, _nupd(nxx, nyy, nzz), 30, 20]
    return _deck("QUARTER2D", 2, mats, nx, ny, 2, [20.0] * nx, [2] * nx, [20.0] * ny, [2] * ny, [10.0, 10.0],
                 [1, 1], [pl], [1, 1], (1, 2, 2, 1, 2, 2), iter_=it)


def _circle_outline(n, radius):
    c = (n - 1) / 2.0
    out = np.zeros((n, n), dtype=bool)
    for i in range(n):
        for j in range(n):
            out[i, j] = np.hypot(i - c, j - c) <= radius
    return out


def full_core_3d(seed=0, nout=2000):
    """17x17 assemblies with reflector corners, 20 fuel layers + reflector top and bottom, 2 groups."""
    rng = np.random.default_rng(1000 + seed)
    fuels = [_fuel2(rng) for _ in range(3)]
    rodded = []
    for f in fuels:
        g = dict(f)
        g["sa"] = [f["sa"][0], f["sa"][1] + 0.02]
        rodded.append(g)
    mats = [_mat2(**REFL2)] + [_mat2(**f) for f in fuels] + [_mat2(**f) for f in rodded]
    n = 17
    fuel = _circle_outline(n, 7.2)
    types = rng.integers(0, 3, size=(n, n))
    fuel_pos = np.argwhere(fuel)
    rods = fuel_pos[rng.choice(len(fuel_pos), size=8, replace=False)]
    rodmask = np.zeros((n, n), dtype=bool)
    rodmask[rods[:, 0], rods[:, 1]] = True
    refl = np.ones((n, n), dtype=int)
    unrod = np.where(fuel, 2 + types, 1)
    rod = np.where(fuel & rodmask, 5 + types, unrod)
    planars = [refl, unrod, rod]
    zpln = [1] + [2] * 12 + [3] * 8 + [1]
    nxx = nyy = 34
    nzz = 22
    it = [nout, 2, "1.0e-5", "1.0e-5", 5, _nupd(nxx, nyy, nzz), 30, 20]
    return _deck("FULL3D", 2, mats, n, n, 22, [20.0] * n, [2] * n, [20.0] * n, [2] * n, [20.0] * 22, [1] * 22,
                 planars, zpln, (1, 1, 1, 1, 1, 1), iter_=it)


def _mat4(D, sa, nuf, ss, chi):
    rows = []
    for g in range(4):
        rows.append([1.0 / (3.0 * D[g]), sa[g], nuf[g], nuf[g] / NU, chi[g]] + list(ss[g]))
    return rows


def core_4g(seed=0, nout=2000, planes=80):
    """17x17 assemblies of 4x4 nodes, 80 planes of 5 cm, 4 groups, down-scatter only.

    planes = 80 / zdiv with zdiv in {1, 2, 4} gives the same core with coarser
    axial nodes (used for smaller profiling cases)."""
    rng = np.random.default_rng(2000 + seed)
    D = np.geomspace(2.0, 0.35, 4)
    chi = (0.75, 0.25, 0.0, 0.0)
    sa_mean = np.array([0.010, 0.010, 0.090, 0.090])
    nuf_mean = np.array([0.006, 0.006, 0.130, 0.130])

    def down(rng):
        ss = np.zeros((4, 4))
        for g in range(4):
            for h in range(g + 1, 4):
                ss[g, h] = rng.uniform(0.001, 0.05)
        return ss

    fuels = []
    for _ in range(3):
        sa = sa_mean * rng.lognormal(0.0, 0.1, 4)
        nuf = nuf_mean * rng.lognormal(0.0, 0.1, 4)
        fuels.append(_mat4(D, sa, nuf, down(rng), chi))
    refl = _mat4(D * 0.9, np.array([0.0005, 0.001, 0.01, 0.02]), np.zeros(4), down(rng), (0.0, 0.0, 0.0, 0.0))
    mats = [refl] + fuels
    n = 17
    fuel = _circle_outline(n, 7.2)
    types = rng.integers(0, 3, size=(n, n))
    pl = np.where(fuel, 2 + types, 1)
    zdiv = planes // 20
    if zdiv not in (1, 2, 4) or zdiv * 20 != planes:
        raise ValueError("planes must be 20, 40 or 80")
    nxx = nyy = 68
    nzz = planes
    it = [nout, 2, "1.0e-5", "1.0e-5", 5, _nupd(nxx, nyy, nzz), 30, 20]
    return _deck("CORE4G", 4, mats, n, n, 20, [20.0] * n, [4] * n, [20.0] * n, [4] * n, [20.0] * 20, [zdiv] * 20,
                 [pl], [1] * 20, (1, 1, 1, 1, 1, 1), iter_=it)


def _split_nodes(n, max_asm=33):
    """Assembly divisions (2 or 3 nodes) summing to n with at most max_asm assemblies."""
    nx = min(max_asm, max(2, n // 2))
    div = [n // nx] * nx
    for q in range(n - sum(div)):
        div[q] += 1
    return div


def batch_member(seed, index, zref=True, zsize=10.0, nupd=100):
    """One member of the batched workload: drawn radial/axial size, 1% lognormal XS perturbation.

    zref: the first and last axial nodes are reflector (as in the 3D full
    core); zsize: axial node height in cm.  nupd: nodal update interval.
    The default interval ceil((nxx+nyy+nzz)/2.5) starts the nodal updates
    before the CMFD flux of these larger cores has settled, and the
    reference's two-node iteration then diverges on about one core in five
    (ndmax > 1e3, mod_nodal.f90:131-142); 100 outers avoid that."""
    rng = np.random.default_rng([3000 + seed, index])
    nr = int(rng.integers(20, 69))
    nzn = int(rng.integers(10, 41))
    base = np.random.default_rng(1000 + seed)
    fuels = [_fuel2(base) for _ in range(3)]

    def pert(f):
        q = dict(D=tuple(d * rng.lognormal(0, 0.01) for d in f["D"]),
                 sa=[s * rng.lognormal(0, 0.01) for s in f["sa"]],
                 nuf=tuple(s * rng.lognormal(0, 0.01) for s in f["nuf"]),
                 s12=f["s12"] * rng.lognormal(0, 0.01))
        return q

    mats = [_mat2(**pert(REFL2))] + [_mat2(**pert(f)) for f in fuels]
    div = _split_nodes(nr)
    nx = len(div)
    # cylindrical outline: fuel inside the circle, one ring of reflector
    # assemblies, no nodes beyond (a square box with thick reflector corners
    # drives the reference's two-node iteration unstable on the larger cores)
    rad = 0.5 * nx
    fuel = _circle_outline(nx, rad - 1.0)
    core = _circle_outline(nx, rad + 0.25)
    types = rng.integers(0, 3, size=(nx, nx))
    pl = np.where(fuel, 2 + types, np.where(core, 1, 0))
    size = [10.0 * d for d in div]
    it = [2000, 2, "1.0e-5", "1.0e-5", 5, nupd, 30, 20]
    planars = [pl]
    zpln = [1] * nzn
    if zref:
        planars.append(np.where(pl > 0, 1, 0))
        zpln[0] = zpln[-1] = 2
    return _deck(f"BATCH{index}", 2, mats, nx, nx, nzn, size, div, size, div, [zsize] * nzn, [1] * nzn,
                 planars, zpln, (1, 1, 1, 1, 1, 1), iter_=it)


def batch_member_stated(seed, index):
    """A member of the batched workload with the config-1 cross-section sets
    as stated for it, and the reference's default nodal-update interval.

    Radial nodes U{20..68} (assemblies of 2 or 3 nodes, corner reflector by
    the circle test as the full core), axial nodes U{10..40} of 20 cm with a
    reflector node at the bottom and top; the materials of full_core_3d
    (reflector, three fuel types, their rodded variants with sigma_a2 +
    0.02) each scaled per parameter by an independent lognormal factor
    (sigma 1%); the rodded region is 8 seeded fuel assemblies over the top
    40% of the fuel planes; nupd = ceil((nxx + nyy + nzz) / 2.5)
    (mod_io.f90:1363).  No draw is filtered: members on which the
    reference's two-node iteration diverges stay in the batch."""
    rng = np.random.default_rng([5000 + seed, index])
    nr = int(rng.integers(20, 69))
    nzn = int(rng.integers(10, 41))
    base = np.random.default_rng(1000 + seed)
    fuels = [_fuel2(base) for _ in range(3)]

    def pert(f):
        return dict(D=tuple(d * rng.lognormal(0, 0.01) for d in f["D"]),
                    sa=[s * rng.lognormal(0, 0.01) for s in f["sa"]],
                    nuf=tuple(s * rng.lognormal(0, 0.01) for s in f["nuf"]),
                    s12=f["s12"] * rng.lognormal(0, 0.01))

    rodded = []
    for f in fuels:
        g = dict(f)
        g["sa"] = [f["sa"][0], f["sa"][1] + 0.02]
        rodded.append(g)
    mats = [_mat2(**pert(REFL2))] + [_mat2(**pert(f)) for f in fuels] + [_mat2(**pert(f)) for f in rodded]
    div = _split_nodes(nr)
    n = len(div)
    fuel = _circle_outline(n, 7.2 / 17.0 * n)
    types = rng.integers(0, 3, size=(n, n))
    fuel_pos = np.argwhere(fuel)
    nrod = min(8, len(fuel_pos))
    rods = fuel_pos[rng.choice(len(fuel_pos), size=nrod, replace=False)]
    rodmask = np.zeros((n, n), dtype=bool)
    rodmask[rods[:, 0], rods[:, 1]] = True
    refl = np.ones((n, n), dtype=int)
    unrod = np.where(fuel, 2 + types, 1)
    rod = np.where(fuel & rodmask, 5 + types, unrod)
    nfuel = nzn - 2
    ntop = int(round(0.4 * nfuel))
    zpln = [1] + [2] * (nfuel - ntop) + [3] * ntop + [1]
    size = [10.0 * d for d in div]
    it = [2000, 2, "1.0e-5", "1.0e-5", 5, _nupd(sum(div), sum(div), nzn), 30, 20]
    return _deck(f"BATCHS{index}", 2, mats, n, n, nzn, size, div, size, div, [20.0] * nzn, [1] * nzn,
                 [refl, unrod, rod], zpln, (1, 1, 1, 1, 1, 1), iter_=it)


def _changes2(rows):
    """Feedback-card records of 2-group materials: per material two rows
    sigtr siga nuf sigf sigs(g->1) sigs(g->2)."""
    return [" ".join(_fmt(v) for v in row) for mat in rows for row in mat]


def boron_search_3d(seed=0, n=17, planes=20, rbcon=1000.0):
    """Critical boron search on a 3D full core (mode BCSEARCH).

    n x n assemblies of 2x2 nodes (fuel inside a circle of radius 0.42 n,
    reflector outside), `planes` fuel layers of 20 cm between reflector
    layers, 3 fuel types, 2 groups, SANM.  Cross sections are given at the
    reference boron concentration rbcon; the feedback cards carry boron
    worth (about 9 pcm/ppm), fuel and moderator temperatures and coolant
    density away from their references, and two control-rod banks of four
    assemblies each, at 120 and 200 of 228 steps over the fuel height (tips
    inside nodes, so the volume-weighted rodded nodes are exercised)."""
    rng = np.random.default_rng(2000 + seed)
    fuels = [_fuel2(rng) for _ in range(3)]

    def borated(f):   # the tables hold rbcon's absorption on top of the unborated values
        g = dict(f)
        g["sa"] = [f["sa"][0] + rbcon * 1.9e-7, f["sa"][1] + rbcon * 1.03e-5]
        return g

    mats = [_mat2(**borated(REFL2))] + [_mat2(**borated(f)) for f in fuels]
    fuel = _circle_outline(n, 0.42 * n)
    types = rng.integers(0, 3, size=(n, n))
    fuel_pos = np.argwhere(fuel)
    rods = fuel_pos[rng.choice(len(fuel_pos), size=8, replace=False)]
    refl = np.ones((n, n), dtype=int)
    unrod = np.where(fuel, 2 + types, 1)
    nz = planes + 2
    zpln = [1] + [2] * planes + [1]
    nxx = nyy = 2 * n
    it = [3000, 2, "1.0e-5", "1.0e-5", 5, _nupd(nxx, nyy, nz), 30, 20]
    text = _deck("BCSEARCH3D", 2, mats, n, n, nz, [20.0] * n, [2] * n, [20.0] * n, [2] * n, [20.0] * nz, [1] * nz,
                 [refl, unrod], zpln, (1, 1, 1, 1, 1, 1), iter_=it, mode="BCSEARCH")
    nm = len(mats)
    # control rods: banks 1 and 2, map written north row first
    bank = np.zeros((n, n), dtype=int)
    bank[rods[:4, 0], rods[:4, 1]] = 1
    bank[rods[4:, 0], rods[4:, 1]] = 2
    rod = [[3.7e-3, 2.5e-3, -1.0e-4, -1.0e-4 / NU, 0.0, -3.2e-3],
           [-2.2e-2, 2.56e-2, -2.8e-3, -2.8e-3 / NU, 0.0, 0.0]]
    # 228 steps span the fuel height; bank 1 at step 120, bank 2 at 200
    L = ["%CROD", "2 228", "20.0 " + _fmt(20.0 * planes / 228.0), "120.0 200.0"]
    for j in range(n - 1, -1, -1):
        L.append(" ".join(str(int(bank[i, j])) for i in range(n)))
    L += _changes2([rod] * nm)
    # boron, per ppm (water in every material)
    bor = [[6.1e-8, 1.9e-7, 0.0, 0.0, 0.0, 7.9e-10], [5.2e-6, 1.03e-5, 0.0, 0.0, 0.0, 0.0]]
    L += ["%CBCS", _fmt(rbcon)] + _changes2([bor] * nm)
    zero = [[0.0] * 6, [0.0] * 6]
    # fuel temperature, per sqrt(K): Doppler absorption in the fast group
    ftem = [[0.0, 3.0e-5, 0.0, 0.0, 0.0, 0.0], [0.0, 5.0e-6, -5.0e-6, -5.0e-6 / NU, 0.0, 0.0]]
    L += ["%FTEM", "950.0 900.0"] + _changes2([zero] + [ftem] * (nm - 1))
    # moderator temperature, per K
    mtem = [[-6.0e-5, -3.0e-5, -4.0e-5, -4.0e-5 / NU, 0.0, -1.0e-5], [-5.0e-4, -2.0e-4, -3.0e-4, -3.0e-4 / NU, 0.0, 0.0]]
    L += ["%MTEM", "580.0 575.0"] + _changes2([zero] + [mtem] * (nm - 1))
    # coolant density, per g/cm3
    cden = [[7.5e-2, 2.1e-4, 0.0, 0.0, 0.0, 3.7e-2], [5.3e-1, 7.6e-3, 0.0, 0.0, 0.0, 0.0]]
    L += ["%CDEN", "0.72 0.71"] + _changes2([cden] * nm)
    return text + "\n".join(L) + "\n"


def rod_ejection_3d(seed=0, n=17, planes=20, ttot=0.5, tstep1=0.01, tdiv=0.1, tstep2=0.05, theta=0.5, extr=False):
    """Rod ejection (mode RODEJECT) on the core of boron_search_3d: the same
    geometry, cross sections (at its reference boron, no boron card) and two
    rod banks; bank 1 is ejected from step 120 to 228 at 2280 steps/s (0.05 s),
    bank 2 stays.  Six delayed families, 2-group velocities; theta 0.5
    (Crank-Nicolson); the steady state is brought to k = 1 by KNE1.  extr
    adds %EXTR (the exponential flux extrapolation of trans_calc)."""
    text = boron_search_3d(seed, n=n, planes=planes)
    out, skip = [], False
    for ln in text.splitlines():
        t = ln.strip()
        if t.startswith("%"):
            skip = t[1:] in ("CBCS", "FTEM", "MTEM", "CDEN")
        if not skip:
            out.append(ln)
    text = "\n".join(out).replace("%MODE\nBCSEARCH", "%MODE\nRODEJECT") + "\n"
    L = ["%EJCT",
         "228.0 0.0 2280.0",
         "200.0 0.0 0.0",
         " ".join(_fmt(v) for v in (ttot, tstep1, tdiv, tstep2)),
         "0.000215 0.001424 0.001274 0.002568 0.000748 0.000273",
         "0.0124 0.0305 0.111 0.301 1.14 3.01",
         "2.0e7 2.2e5",
         "%THET", _fmt(theta)]
    if extr:
        L.append("%EXTR")
    return text + "\n".join(L) + "\n"


def small_core(seed=0, ng=2, kern="SANM", nx=4, ny=4, nz=3, xdiv=2, ydiv=2, zdiv=1, ragged=True, adf=False,
               bc=None, mode="FORWARD", nout=3000):
    """A small core for parity tests: ragged outline, optional ADFs, random BCs, ng groups."""
    rng = np.random.default_rng(seed)
    nmat = 3
    mats = []
    for m in range(nmat):
        D = np.geomspace(1.5, 0.4, ng) * rng.uniform(0.9, 1.1, ng)
        sa = np.where(np.arange(ng) < ng / 2, 0.01, 0.09) * rng.uniform(0.8, 1.2, ng)
        nuf = (np.where(np.arange(ng) < ng / 2, 0.006, 0.13) * rng.uniform(0.8, 1.2, ng)) if m > 0 else np.zeros(ng)
        chi = np.zeros(ng)
        chi[0] = 1.0 if ng == 1 else 0.8
        if ng > 1:
            chi[1] = 0.2
        if ng == 1:
            sa = sa * 0.0 + 0.02
            nuf = nuf * 0.0 + (0.025 if m > 0 else 0.0)
        ss = np.zeros((ng, ng))
        for g in range(ng):
            for h in range(ng):
                if h > g:
                    ss[g, h] = rng.uniform(0.005, 0.03)
                elif h < g and rng.uniform() < 0.3:
                    ss[g, h] = rng.uniform(0.0, 0.002)   # some up-scatter
        rows = [[1.0 / (3.0 * D[g]), sa[g], nuf[g], nuf[g] / NU, chi[g]] + list(ss[g]) for g in range(ng)]
        mats.append(rows)
    pl = np.zeros((nx, ny), dtype=int)
    for i in range(nx):
        for j in range(ny):
            pl[i, j] = 1 if (i == nx - 1 or j == ny - 1) else int(rng.integers(2, 4))
    if ragged and nx >= 3 and ny >= 3:
        pl[nx - 1, ny - 1] = 0          # cut the outer corner
    if bc is None:
        bc = tuple(int(v) for v in rng.integers(0, 3, 6))
    nxx, nyy, nzz = nx * xdiv, ny * ydiv, nz * zdiv
    it = [nout, 2, "1.0e-5", "1.0e-5", 5, _nupd(nxx, nyy, nzz), 30, 20]
    adf_rows = None
    if adf:
        adf_rows = [[list(rng.uniform(0.85, 1.15, 6)) for _ in range(ng)] for _ in range(nmat)]
    return _deck("SMALL", ng, mats, nx, ny, nz, [15.0] * nx, [xdiv] * nx, [15.0] * ny, [ydiv] * ny,
                 [20.0] * nz, [zdiv] * nz, [pl], [1] * nz, bc, kern=kern, iter_=it, adf=adf_rows, mode=mode)


CONFIGS = {
    "quarter_core_2d": quarter_core_2d,
    "full_core_3d": full_core_3d,
    "core_4g": core_4g,
}
