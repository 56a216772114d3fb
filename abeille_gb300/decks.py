"""Synthetic multigroup decks for the benchmark configurations.

Every deck is generated from fixed seeds (cross sections from seed 1), so a
configuration means the same problem on every machine.  Group 0 is the fastest
group, as in the reference's c5g7 deck; energy bounds are the labels [0, 1, ..., G].

Geometry follows the reference's own lattice decks (input_files/c5g7.yaml): the
root universe is a rectilinear lattice whose outer universe holds the box cell
bounded by the boundary-condition surfaces.

  config0  17x17 pin lattice, pitch 1.26, fuel radius 0.54, reflective x/y,
           infinite in z; fuel + moderator, 7 groups; k-eigenvalue, delta
           tracking; 17x17x1 collision flux tally.
  config1  51x51 pins, 200 cm tall in 10 axial zones bounded by z-planes
           (root universe of 10 zone cells, each filled with a 51x51 lattice),
           vacuum top/bottom, reflective sides, a 5x5 water-gap box in the
           centre; 7 groups; 51x51x20 collision flux tally.
  config2  17x17 pins with fuel/gap/clad rings (r = 0.41/0.42/0.475), 8 fuel
           compositions drawn per pin, 70 groups, upscatter in the lowest 10
           groups, P1 scattering with mean cosine in [0, 0.3]; 100 cm tall,
           vacuum top/bottom; 100x100x50 track-length flux tally.
  config3  non-multiplying fixed-source slab boxes (see fixed_source_problem).
  quadrics every other surface kind of the path in one cell universe: a fuel
           sphere, a fuel x-cylinder rod, a water y-cylinder rod, moderator
           split by a general plane, inside a vacuum sphere cut by a
           reflective general plane; 7 groups; collision and track-length
           flux tallies.
"""
import numpy as np

from .problem import ProblemBuilder

PITCH = 1.26


def _downscatter_matrix(rng, sig_s, frac_down, G, upscatter_from=None, up_frac=0.0):
    """Row g: (1-frac_down) in-group, frac_down spread over lower groups with
    geometric weights; optional upscatter inside the thermal block."""
    S = np.zeros((G, G))
    for g in range(G):
        below = np.arange(g + 1, G)
        if below.size == 0:
            S[g, g] = sig_s[g]
            continue
        w = 0.35 ** (below - g - 1) * (0.8 + 0.4 * rng.random(below.size))
        w /= w.sum()
        fd = frac_down
        fu = 0.0
        if upscatter_from is not None and g > upscatter_from:
            fu = up_frac
            # keep the in-group element non-negative (the reference refuses
            # negative scattering components, src/mg_nuclide.cpp:628-634)
            if fd + fu > 0.99:
                fd = 0.99 - fu
            above = np.arange(upscatter_from, g)
            wu = 0.5 ** (g - above - 1) * (0.8 + 0.4 * rng.random(above.size))
            wu /= wu.sum()
            S[g, above] = sig_s[g] * fu * wu
        S[g, g] = sig_s[g] * (1.0 - fd - fu)
        S[g, below] = sig_s[g] * fd * w
    return S


def seven_group_xs(seed=1):
    """The 7-group synthetic set: moderator, fuel, water gap."""
    G = 7
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 1.0, G)
    # moderator: sigma_t 0.2 -> 3.0 /cm, scattering ratio 0.90 -> 0.99, 95 % downscatter
    mt = 0.2 + 2.8 * t
    mc = 0.90 + 0.09 * t
    ms = mt * mc
    mS = _downscatter_matrix(rng, ms, 0.95, G)
    ms_row = mS.sum(axis=1)
    mod = dict(total=mt, absorption=mt - ms_row, scatter=mS)
    # fuel: sigma_t 0.3 -> 1.5, nu*sigma_f/sigma_t 0.02 -> 0.3, nu = 2.5, chi (0.6, 0.35, 0.05)
    ft = 0.3 + 1.2 * t
    nusf = (0.02 + 0.28 * t) * ft
    nu = np.full(G, 2.5)
    fis = nusf / nu
    cap = 0.4 * fis + 0.01 * ft
    fa = fis + cap
    fS = _downscatter_matrix(rng, ft - fa, 0.5, G)
    fuel = dict(total=ft, absorption=ft - fS.sum(axis=1), scatter=fS, fission=fis, nu=nu,
                chi=[0.6, 0.35, 0.05, 0.0, 0.0, 0.0, 0.0])
    # water gap: the moderator's scattering with 0.2x its absorption
    wa = 0.2 * mod["absorption"]
    water = dict(total=ms_row + wa, absorption=wa, scatter=mS)
    return fuel, mod, water


def _box_outer(b, half_x, half_y, zlo=None, zhi=None, xy_bc="reflective", z_bc="vacuum", sid0=100, cid=100,
               uid=100, mat=None):
    b.surface("xplane", sid0 + 1, x0=-half_x, boundary=xy_bc)
    b.surface("xplane", sid0 + 2, x0=half_x, boundary=xy_bc)
    b.surface("yplane", sid0 + 3, y0=-half_y, boundary=xy_bc)
    b.surface("yplane", sid0 + 4, y0=half_y, boundary=xy_bc)
    reg = f"+{sid0 + 1} & -{sid0 + 2} & +{sid0 + 3} & -{sid0 + 4}"
    if zlo is not None:
        b.surface("zplane", sid0 + 5, z0=zlo, boundary=z_bc)
        b.surface("zplane", sid0 + 6, z0=zhi, boundary=z_bc)
        reg += f" & +{sid0 + 5} & -{sid0 + 6}"
    b.cell(cid, reg, material=mat)
    b.cell_universe(uid, [cid])
    return uid


def config0(nparticles=10000, precision="fp64", tracking="delta-tracking"):
    fuel, mod, _ = seven_group_xs()
    b = ProblemBuilder(7, np.arange(8.0), nparticles=nparticles, precision=precision, tracking=tracking)
    b.material(1, **fuel)
    b.material(2, **mod)
    b.surface("zcylinder", 1, x0=0.0, y0=0.0, r=0.54)
    b.cell(1, "-1", material=1)
    b.cell(2, "+1", material=2)
    half = 17 * PITCH / 2
    outer = _box_outer(b, half, half, mat=2)
    b.cell_universe(1, [1, 2])
    b.rect_lattice(10, [17, 17, 1], [PITCH, PITCH, 1.0e6], [0.0, 0.0, 0.0], [1] * (17 * 17), outer=outer)
    b.set_root(10)
    b.mesh_tally([17, 17, 1], [-half, -half, -5.0e5], [half, half, 5.0e5], "collision", "flux", [0.0, 7.0])
    b.set_entropy([-half, -half, -5.0e5], [half, half, 5.0e5], [17, 17, 1])
    b.source("box", low=[-half, -half, -10.0], hi=[half, half, 10.0], energy=0.5, fissile_only=True)
    return b


def config1(nparticles=1000000, precision="fp64", tracking="delta-tracking"):
    fuel, mod, water = seven_group_xs()
    b = ProblemBuilder(7, np.arange(8.0), nparticles=nparticles, precision=precision, tracking=tracking)
    b.material(1, **fuel)
    b.material(2, **mod)
    b.material(3, **water)
    # pins: fuel cylinder in moderator; water-gap tiles: one water cell
    b.surface("zcylinder", 1, x0=0.0, y0=0.0, r=0.54)
    b.surface("zcylinder", 2, x0=0.0, y0=0.0, r=100.0)
    b.cell(1, "-1", material=1)
    b.cell(2, "+1", material=2)
    b.cell(3, "-2", material=3)
    b.cell_universe(1, [1, 2])
    b.cell_universe(2, [3])
    half = 51 * PITCH / 2
    # boundary planes: reflective sides, vacuum top and bottom
    b.surface("xplane", 101, x0=-half, boundary="reflective")
    b.surface("xplane", 102, x0=half, boundary="reflective")
    b.surface("yplane", 103, y0=-half, boundary="reflective")
    b.surface("yplane", 104, y0=half, boundary="reflective")
    zs = [-100.0 + 20.0 * k for k in range(11)]  # 11 planes bound 10 axial zones
    for k, z in enumerate(zs):
        b.surface("zplane", 110 + k, z0=z, boundary="vacuum" if k in (0, 10) else "normal")
    tiles = []
    for i in range(51):        # yaml order: nx runs down the list, ny fastest
        for j in range(51):
            tiles.append(2 if (abs(i - 25) <= 2 and abs(j - 25) <= 2) else 1)
    # root: one cell per axial zone, bounded by z-planes, each filled with its
    # own copy of the 51x51 lattice.  The lattice copy takes the zone cell's
    # id, so the reference's re-descent by the cell pad's id
    # (universe_id_to_indx[tree.back().id]) lands on that lattice.
    zone_cells = []
    for zone in range(10):
        cid = 200 + zone
        b.rect_lattice(cid, [51, 51, 1], [PITCH, PITCH, 20.0], [0.0, 0.0, zs[zone] + 10.0], tiles)
        b.cell(cid, f"+101 & -102 & +103 & -104 & +{110 + zone} & -{111 + zone}", universe=cid)
        zone_cells.append(cid)
    b.cell_universe(300, zone_cells)
    b.set_root(300)
    b.mesh_tally([51, 51, 20], [-half, -half, -100.0], [half, half, 100.0], "collision", "flux", [0.0, 7.0])
    b.set_entropy([-half, -half, -100.0], [half, half, 100.0], [17, 17, 10])
    b.source("box", low=[-half, -half, -100.0], hi=[half, half, 100.0], energy=0.5, fissile_only=True)
    return b


def seventy_group_xs(seed=1, nfuel=8):
    G = 70
    rng = np.random.default_rng(seed)
    mats = []

    def base(frac_down, scat_ratio, up_frac, fissile):
        tot = np.exp(rng.uniform(np.log(0.1), np.log(10.0), G))
        sig_s = tot * scat_ratio
        S = _downscatter_matrix(rng, sig_s, frac_down, G, upscatter_from=60, up_frac=up_frac)
        P1 = rng.uniform(0.0, 0.3, (G, G))
        d = dict(total=tot, absorption=tot - S.sum(axis=1), scatter=S, legendre={1: P1})
        if fissile:
            nusf = rng.uniform(0.02, 0.3, G) * tot * (1.0 - scat_ratio) / 0.3
            nu = np.full(G, 2.45)
            fis = nusf / nu
            d["absorption"] = np.maximum(d["absorption"], fis * 1.1)
            d["total"] = S.sum(axis=1) + d["absorption"]
            chi = np.zeros(G)
            chi[:12] = np.exp(-np.arange(12) / 3.0)
            d.update(fission=fis, nu=nu, chi=chi / chi.sum())
        return d

    for f in range(nfuel):
        mats.append(base(0.5, 0.7, 0.05, True))
    mats.append(base(0.3, 0.5, 0.0, False))    # gap
    mats.append(base(0.6, 0.8, 0.05, False))   # clad
    mats.append(base(0.95, 0.97, 0.15, False))  # moderator
    return mats


def quadrics(nparticles=4096, precision="fp64", tracking="delta-tracking", legendre=False, cap="reflective"):
    """Spheres, general planes (normals off the axes, one of them a boundary
    condition, reflective by default) and x/y-cylinders, the surface kinds the
    lattice configurations do not use (src/sphere.cpp, src/plane.cpp,
    src/xcylinder.cpp, src/ycylinder.cpp).  With `legendre`, the moderator
    scatters with mean cosine 0.2 (a P1 entry), so angle tables are sampled as
    well.

    A reflective general plane is where the reference's own arithmetic is
    most fragile: Plane::distance (src/plane.cpp:47-59) compares the distance,
    not the position, with SURFACE_COINCIDENT, so a particle reflected at
    grazing incidence and left a rounding error on the far side of the plane
    can find it again a few 1e-12 cm away and be lost.  Runs of very many
    FP64 histories use `cap="vacuum"`."""
    fuel, mod, water = seven_group_xs()
    b = ProblemBuilder(7, np.arange(8.0), nparticles=nparticles, precision=precision, tracking=tracking)
    b.material(1, **fuel)
    if legendre:
        # P1 entries are mean scattering cosines (pdf 1/2 + 3/2 mu_bar mu)
        mod = dict(mod, legendre={1: 0.2 * (np.asarray(mod["scatter"]) > 0)})
    b.material(2, **mod)
    b.material(3, **water)
    b.surface("sphere", 1, x0=0.0, y0=0.0, z0=0.0, r=3.0)
    b.surface("xcylinder", 2, y0=6.0, z0=3.0, r=1.5)
    b.surface("ycylinder", 3, x0=-6.0, z0=-3.0, r=1.5)
    b.surface("plane", 4, A=0.6, B=0.48, C=0.64, D=1.5)
    b.surface("sphere", 5, x0=0.0, y0=0.0, z0=0.0, r=11.0, boundary="vacuum")
    b.surface("plane", 6, A=0.3, B=-0.4, C=0.8660254037844386, D=5.0, boundary=cap)
    b.cell(1, "-1", material=1)
    b.cell(2, "-2 & -5 & -6", material=1)
    b.cell(3, "-3 & -5 & -6", material=3)
    b.cell(4, "+1 & +2 & +3 & -4 & -5 & -6", material=2)
    b.cell(5, "+1 & +2 & +3 & +4 & -5 & -6", material=3)
    b.cell_universe(1, [1, 2, 3, 4, 5])
    b.set_root(1)
    b.mesh_tally([11, 11, 11], [-11.0, -11.0, -11.0], [11.0, 11.0, 11.0], "collision", "flux", [0.0, 7.0])
    b.mesh_tally([11, 11, 11], [-11.0, -11.0, -11.0], [11.0, 11.0, 11.0], "track-length", "flux", [0.0, 7.0])
    b.set_entropy([-11.0, -11.0, -11.0], [11.0, 11.0, 11.0], [8, 8, 8])
    b.source("box", low=[-3.0, -3.0, -3.0], hi=[3.0, 3.0, 3.0], energy=0.5, fissile_only=True)
    return b


def config2(nparticles=2000000, precision="fp64", tracking="surface-tracking"):
    mats = seventy_group_xs()
    G = 70
    b = ProblemBuilder(G, np.arange(G + 1.0), nparticles=nparticles, precision=precision, tracking=tracking)
    for i, m in enumerate(mats):
        b.material(i + 1, **m)
    b.surface("zcylinder", 1, x0=0.0, y0=0.0, r=0.41)
    b.surface("zcylinder", 2, x0=0.0, y0=0.0, r=0.42)
    b.surface("zcylinder", 3, x0=0.0, y0=0.0, r=0.475)
    gap, clad, moder = 9, 10, 11
    rng = np.random.default_rng(2)
    comps = rng.integers(0, 8, 17 * 17)
    for f in range(8):
        c0 = 10 * (f + 1)
        b.cell(c0 + 1, "-1", material=f + 1)
        b.cell(c0 + 2, "+1 & -2", material=gap)
        b.cell(c0 + 3, "+2 & -3", material=clad)
        b.cell(c0 + 4, "+3", material=moder)
        b.cell_universe(f + 1, [c0 + 1, c0 + 2, c0 + 3, c0 + 4])
    half = 17 * PITCH / 2
    outer = _box_outer(b, half, half, -50.0, 50.0, mat=moder)
    b.rect_lattice(200, [17, 17, 1], [PITCH, PITCH, 100.0], [0.0, 0.0, 0.0], [int(c) + 1 for c in comps],
                   outer=outer)
    b.set_root(200)
    b.mesh_tally([100, 100, 50], [-half, -half, -50.0], [half, half, 50.0], "track-length", "flux",
                 [0.0, float(G)])
    b.set_entropy([-half, -half, -50.0], [half, half, 50.0], [17, 17, 5])
    b.source("box", low=[-half, -half, -50.0], hi=[half, half, 50.0], energy=0.5, fissile_only=True)
    return b


def fixed_source_problem(index, seed=3, precision="mixed", nparticles=None, tracking="delta-tracking", batches=10):
    """One config-3 problem: a box of 1-4 slabs along x (thickness log-uniform
    1-50 cm), G in {7, 22, 44}, sigma_t in [0.05, 5], scattering ratio in
    [0.3, 0.99], isotropic point source at the centre in group 0, 20x20x20
    collision flux tally, vacuum on every side.  Histories log-uniform 1e3-1e5
    in total, run as `batches` batches of nparticles = total / batches (at
    least 1) each; `nparticles` overrides the per-batch count."""
    rng = np.random.default_rng([seed, index])
    G = int(rng.choice([7, 22, 44]))
    nl = int(rng.integers(1, 5))
    th = np.exp(rng.uniform(np.log(1.0), np.log(50.0), nl))
    total = np.exp(rng.uniform(np.log(1e3), np.log(1e5)))
    hist = max(1, int(round(total / batches)))
    if nparticles is not None:
        hist = nparticles
    width = th.sum()
    b = ProblemBuilder(G, np.arange(G + 1.0), mode="fixed-source", nparticles=hist, precision=precision,
                       tracking=tracking, seed=1000003 * (index + 1))
    for l in range(nl):
        tot = rng.uniform(0.05, 5.0, G)
        c = rng.uniform(0.3, 0.99, G)
        S = _downscatter_matrix(rng, tot * c, 0.7, G)
        b.material(l + 1, total=tot, absorption=tot - S.sum(axis=1), scatter=S)
    x = -width / 2
    b.surface("xplane", 1, x0=x, boundary="vacuum")
    for l in range(nl):
        x += th[l]
        b.surface("xplane", l + 2, x0=x, boundary="vacuum" if l == nl - 1 else "normal")
    hy = width / 2
    b.surface("yplane", 50, y0=-hy, boundary="vacuum")
    b.surface("yplane", 51, y0=hy, boundary="vacuum")
    b.surface("zplane", 52, z0=-hy, boundary="vacuum")
    b.surface("zplane", 53, z0=hy, boundary="vacuum")
    for l in range(nl):
        b.cell(l + 1, f"+{l + 1} & -{l + 2} & +50 & -51 & +52 & -53", material=l + 1)
    b.cell_universe(1, list(range(1, nl + 1)))
    b.set_root(1)
    b.mesh_tally([20, 20, 20], [-width / 2, -hy, -hy], [width / 2, hy, hy], "collision", "flux",
                 [0.0, float(G)])
    b.source("point", position=[0.0, 0.0, 0.0], energy=0.5)
    return b


CONFIGS = {0: config0, 1: config1, 2: config2}


def from_reference_deck(deck, nparticles=None, precision="fp64", tracking=None):
    """ProblemBuilder from a parsed reference deck (the dict form of an
    input_files/*.yaml multigroup deck: materials, surfaces, cells, universes,
    root-universe, sources, tallies, entropy, settings)."""
    st = deck["settings"]
    G = int(st["ngroups"])
    b = ProblemBuilder(G, [float(e) for e in st["energy-bounds"]],
                       mode={"k-eigenvalue": "k-eigenvalue", "fixed-source": "fixed-source",
                             "branchless-k-eigenvalue": "branchless-k-eigenvalue"}[st["simulation"]],
                       tracking=tracking or st.get("transport", "surface-tracking"), precision=precision,
                       nparticles=nparticles or int(st["nparticles"]),
                       seed=int(st.get("seed", 19073486328125)), stride=int(st.get("stride", 152917)),
                       wgt_cutoff=float(st.get("wgt-cutoff", 0.25)), wgt_survival=float(st.get("wgt-survival", 1.0)),
                       wgt_split=float(st.get("wgt-split", 2.0)), sampling_xs_ratio=deck.get("sampling-xs-ratio"),
                       branchless_material=bool(st.get("branchless-material", True)),
                       branchless_splitting=bool(st.get("branchless-splitting", False)),
                       branchless_combing=bool(st.get("branchless-combing", True)),
                       # the global stream draws a plot colour for every cell and every
                       # material without one while the deck is read (src/cell.cpp:445-448,
                       # src/material.cpp:440-449): 3 canonical draws of 2 outputs each
                       global_rng_skip=6 * (len(deck["cells"]) + sum(
                           1 for m in deck["materials"]
                           if not (isinstance(m.get("color"), list) and len(m["color"]) == 3))))
    if st.get("cancellation", False):
        # settings::regional_cancellation (src/parser.cpp:805-813)
        raise ValueError("regional cancellation is outside the multigroup transport path")
    for m in deck["materials"]:
        leg = {l: m[f"P{l}"] for l in range(1, 6) if f"P{l}" in m}
        b.material(int(m["id"]), total=m["total"], absorption=m["absorption"], scatter=m["scatter"],
                   fission=m.get("fission"), nu=m.get("nu"), chi=m.get("chi"), legendre=leg or None)
    for s in deck["surfaces"]:
        kw = {k: v for k, v in s.items() if k not in ("type", "id", "boundary", "name")}
        b.surface(s["type"], int(s["id"]), boundary=s.get("boundary", "normal"), **kw)
    for c in deck["cells"]:
        b.cell(int(c["id"]), c["region"], material=c.get("material"), universe=c.get("universe"))
    for u in deck["universes"]:
        if "cells" in u:
            b.cell_universe(int(u["id"]), [int(x) for x in u["cells"]])
        else:
            b.rect_lattice(int(u["id"]), u["shape"], u["pitch"], u["origin"], u["universes"], u.get("outer"))
    b.set_root(int(deck["root-universe"]))
    for s in deck.get("sources", []):
        sp = s["spatial"]
        kind = sp["type"]
        en = s["energy"]
        if en["type"] != "mono-energetic":
            raise ValueError("only mono-energetic sources are in the multigroup path")
        dr = s["direction"]
        b.source(kind, position=sp.get("position"), low=sp.get("low"), hi=sp.get("hi"),
                 direction="isotropic" if dr["type"] == "isotropic" else "mono-directional",
                 direction_vector=dr.get("direction"), energy=float(en["energy"]), weight=float(s["weight"]),
                 # read at the source entry, as src/source.cpp:104-110 does (a
                 # `fissile-only` inside `spatial`, as input_files/c5g7.yaml:321
                 # has it, is not read by the reference)
                 fissile_only=bool(s.get("fissile-only", False)))
    for t in deck.get("tallies", []):
        b.mesh_tally(t["shape"], t["low"], t["hi"], t.get("estimator", "collision"), t.get("quantity", "flux"),
                     t.get("energy-bounds"))
    if "entropy" in deck:
        e = deck["entropy"]
        b.set_entropy(e["low"], e["hi"], e["shape"])
    return b
