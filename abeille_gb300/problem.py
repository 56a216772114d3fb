"""Problem builder: the multigroup deck of the reference, flattened for the C-ABI.

The builder takes the same entities a reference input deck holds (surfaces,
cells with region strings, cell universes, rectilinear lattices, multigroup
materials, mesh tallies, entropy mesh, sources, settings) and produces the
``abx_problem`` struct of include/abeille_gb300.h.  The flattening follows the
reference parser's conventions so a problem means the same thing to both:

* surface tokens are +-(surface index + 1) (src/cell.cpp:301-370);
* regions go through the reference's infix->RPN conversion (src/cell.cpp:250-299);
* universes are indexed in the order the reference parser creates them
  (cells in deck order, each universe-filled cell creating its universe first,
  lattices after their tile and outer universes; src/parser.cpp:177-257,
  src/rect_lattice.cpp:364-424);
* a one-row chi is repeated for every incoming group (src/mg_nuclide.cpp:834-854).
"""
import ctypes as C

import numpy as np

from . import abi


def tokenize_region(region, surface_index):
    """Cell region string -> infix token list (src/cell.cpp:309-360)."""
    out, temp = [], ""

    def flush():
        nonlocal temp
        if temp:
            sid = int(temp)
            if abs(sid) not in surface_index:
                raise ValueError(f"region references unknown surface id {abs(sid)}")
            tok = surface_index[abs(sid)] + 1
            out.append(-tok if sid < 0 else tok)
            temp = ""

    for ch in region:
        if ch in "&()U~":
            flush()
            out.append({"&": abi.OP_INTR, "(": abi.OP_LPAR, ")": abi.OP_RPAR, "U": abi.OP_UNIN,
                        "~": abi.OP_COMP}[ch])
        elif ch in "+-0123456789":
            temp += ch
        elif ch != " ":
            raise ValueError(f"invalid character {ch!r} in region")
    flush()
    return out


def infix_to_rpn(infix):
    """Shunting-yard conversion with the reference's precedences (src/cell.cpp:250-299)."""
    rpn, stack = [], []
    for t in infix:
        if t < abi.OP_UNIN:
            rpn.append(t)
        elif t < abi.OP_RPAR:
            while stack:
                op = stack[-1]
                if op < abi.OP_RPAR and ((t == abi.OP_COMP and t < op) or (t != abi.OP_COMP and t <= op)):
                    rpn.append(stack.pop())
                else:
                    break
            stack.append(t)
        elif t == abi.OP_LPAR:
            stack.append(t)
        else:
            while stack and stack[-1] != abi.OP_LPAR:
                rpn.append(stack.pop())
            if not stack:
                raise ValueError("mismatched parentheses in region")
            stack.pop()
    while stack:
        op = stack.pop()
        if op >= abi.OP_RPAR:
            raise ValueError("mismatched parentheses in region")
        rpn.append(op)
    return rpn


class Built:
    """A flattened problem; keeps the numpy buffers the struct points into alive."""

    def __init__(self, struct, keep, meta):
        self.struct = struct
        self._keep = keep
        self.meta = meta

    @property
    def ptr(self):
        return C.byref(self.struct)


def _ptr(arr, ctype):
    return arr.ctypes.data_as(C.POINTER(ctype))


class ProblemBuilder:
    def __init__(self, ngroups, energy_bounds, mode="k-eigenvalue", tracking="delta-tracking",
                 precision="fp64", nparticles=10000, seed=19073486328125, stride=152917,
                 wgt_cutoff=0.25, wgt_survival=1.0, block_size=0, wgt_split=2.0, sampling_xs_ratio=None,
                 branchless_material=True, branchless_splitting=False, branchless_combing=True,
                 global_rng_skip=None):
        self.G = int(ngroups)
        self.energy_bounds = np.asarray(energy_bounds, dtype=np.float64)
        if self.energy_bounds.shape != (self.G + 1,):
            raise ValueError("energy_bounds must have ngroups+1 entries")
        self.mode, self.tracking, self.precision = mode, tracking, precision
        self.nparticles, self.seed, self.stride = nparticles, seed, stride
        self.wgt_cutoff, self.wgt_survival, self.block_size = wgt_cutoff, wgt_survival, block_size
        self.wgt_split = wgt_split
        # mode "branchless-k-eigenvalue": the branchless collisions of
        # BranchlessPowerIterator (settings branchless-material / -splitting,
        # defaults as src/settings.cpp:87-89)
        self.branchless_material, self.branchless_splitting = bool(branchless_material), bool(branchless_splitting)
        self.branchless_combing = bool(branchless_combing)
        # outputs the reference's global stream draws while reading the deck
        # (plot colours: 6 per cell and per material without one); None: 6 per
        # cell and per material of this builder
        self.global_rng_skip = global_rng_skip
        self.sampling_xs_ratio = None if sampling_xs_ratio is None else [float(x) for x in sampling_xs_ratio]
        self.surfaces, self.cells, self.universes, self.materials = [], [], {}, []
        self.universe_decl = []
        self.tallies, self.sources = [], []
        self.entropy = None
        self.root = None

    # ---------------------------------------------------------------- geometry
    def surface(self, kind, id, boundary="normal", **c):
        keys = {"xplane": ["x0"], "yplane": ["y0"], "zplane": ["z0"], "plane": ["A", "B", "C", "D"],
                "xcylinder": ["y0", "z0", "r"], "ycylinder": ["x0", "z0", "r"], "zcylinder": ["x0", "y0", "r"],
                "sphere": ["x0", "y0", "z0", "r"]}[kind]
        coeff = [float(c.get(k, 0.0)) for k in keys]
        if any(s["id"] == id for s in self.surfaces):
            raise ValueError(f"surface id {id} used twice")
        self.surfaces.append({"kind": kind, "id": id, "bc": boundary, "c": coeff})
        return id

    def cell(self, id, region, material=None, universe=None):
        if (material is None) == (universe is None):
            raise ValueError("a cell has exactly one of material/universe")
        self.cells.append({"id": id, "region": region, "material": material, "universe": universe})
        return id

    def cell_universe(self, id, cells):
        self.universes[id] = {"kind": "cells", "id": id, "cells": list(cells)}
        self.universe_decl.append(id)
        return id

    def rect_lattice(self, id, shape, pitch, origin, universes, outer=None):
        shape = [int(s) for s in shape]
        universes = [int(u) for u in np.asarray(universes).ravel()]
        if len(universes) != shape[0] * shape[1] * shape[2]:
            raise ValueError("lattice universes do not match its shape")
        self.universes[id] = {"kind": "lattice", "id": id, "shape": shape, "pitch": [float(p) for p in pitch],
                              "origin": [float(o) for o in origin], "tiles": universes,
                              "outer": -1 if outer is None else int(outer)}
        self.universe_decl.append(id)
        return id

    def set_root(self, id):
        self.root = id

    # --------------------------------------------------------------- materials
    def material(self, id, total, absorption, scatter, fission=None, nu=None, nu_prompt=None,
                 nu_delayed=None, chi=None, legendre=None, delayed_probabilities=None, decay_constants=None):
        """One multigroup material (src/mg_nuclide.cpp:579-922).  `legendre` is a
        dict {l: GxG matrix} of P_l moments, l in 1..5."""
        G = self.G
        tot = np.asarray(total, float).reshape(G)
        ab = np.asarray(absorption, float).reshape(G)
        sc = np.asarray(scatter, float).reshape(G, G)
        fi = np.zeros(G) if fission is None else np.asarray(fission, float).reshape(G)
        fissile = bool(np.any(fi > 0))
        nup, nud = np.zeros(G), np.zeros(G)
        ch = np.zeros((G, G))
        if fissile:
            if nu is not None:
                nup = np.asarray(nu, float).reshape(G)
            elif nu_prompt is not None and nu_delayed is not None:
                nup = np.asarray(nu_prompt, float).reshape(G)
                nud = np.asarray(nu_delayed, float).reshape(G)
            else:
                raise ValueError(f"material {id}: fissile material needs nu")
            if chi is None:
                raise ValueError(f"material {id}: fissile material needs chi")
            chi = np.asarray(chi, float)
            ch = np.repeat(chi.reshape(1, G), G, axis=0) if chi.size == G else chi.reshape(G, G)
        leg = legendre or {}
        L = max(leg) if leg else 0
        moments = np.zeros((L, G, G))
        for l, m in leg.items():
            if not 1 <= l <= 5:
                raise ValueError("Legendre order must be 1..5")
            moments[l - 1] = np.asarray(m, float).reshape(G, G)
        dp = np.asarray(delayed_probabilities if delayed_probabilities is not None else [], float)
        dc = np.asarray(decay_constants if decay_constants is not None else [], float)
        if dp.shape != dc.shape:
            raise ValueError("delayed probabilities and constants differ in size")
        self.materials.append({"id": id, "data": np.concatenate([tot, ab, fi, nup, nud, ch.ravel(), sc.ravel(),
                                                                 moments.ravel(), dp, dc]),
                               "n_legendre": L, "n_delayed": dp.size, "fissile": fissile})
        return id

    # ------------------------------------------------------- tallies, sources
    def mesh_tally(self, shape, low, hi, estimator="collision", quantity="flux", energy_bounds=None):
        eb = self.energy_bounds if energy_bounds is None else np.asarray(energy_bounds, float)
        self.tallies.append({"shape": [int(s) for s in shape], "low": [float(v) for v in low],
                             "hi": [float(v) for v in hi], "est": abi.EST[estimator],
                             "q": abi.QUANTITY[quantity], "eb": eb})
        return len(self.tallies) - 1

    def set_entropy(self, low, hi, shape):
        self.entropy = {"low": [float(v) for v in low], "hi": [float(v) for v in hi], "shape": [int(s) for s in shape]}

    def source(self, spatial="point", position=None, low=None, hi=None, direction="isotropic",
               direction_vector=None, energy=1.0, weight=1.0, fissile_only=False):
        s = abi.Source()
        s.spatial = abi.SPATIAL[spatial]
        s.direction = abi.DIRECTION[direction]
        s.energy = 0
        s.fissile_only = int(bool(fissile_only))
        s.weight = float(weight)
        lo = position if spatial == "point" else low
        for a in range(3):
            s.low[a] = float(lo[a])
            s.hi[a] = float(hi[a]) if hi is not None else float(lo[a])
            s.dir[a] = float(direction_vector[a]) if direction_vector is not None else (1.0 if a == 0 else 0.0)
        s.energy_value = float(energy)
        self.sources.append(s)

    # ------------------------------------------------------------ deck output
    def to_deck(self, ngenerations=None, nignored=None):
        """The problem as a reference-format deck dictionary (write it with
        deck.dump_yaml), so the reference can run the same problem."""
        G = self.G
        inv = {v: k for k, v in abi.SURF.items()}
        keys = {"xplane": ["x0"], "yplane": ["y0"], "zplane": ["z0"], "plane": ["A", "B", "C", "D"],
                "xcylinder": ["y0", "z0", "r"], "ycylinder": ["x0", "z0", "r"], "zcylinder": ["x0", "y0", "r"],
                "sphere": ["x0", "y0", "z0", "r"]}
        mats = []
        for m in self.materials:
            d = m["data"]
            if m["n_delayed"]:
                raise ValueError("delayed-neutron data is not written to decks")
            o = 0
            tot, ab, fi, nup, nud = (d[o + k * G:o + (k + 1) * G] for k in range(5))
            o = 5 * G
            chi = d[o:o + G * G].reshape(G, G)
            sc = d[o + G * G:o + 2 * G * G].reshape(G, G)
            e = {"id": m["id"], "total": tot.tolist(), "absorption": ab.tolist(), "scatter": sc.tolist()}
            if m["fissile"]:
                e["fission"] = fi.tolist()
                e["nu"] = (nup + nud).tolist()
                e["chi"] = [chi[0].tolist()] if np.all(chi == chi[0]) else chi.tolist()
            mom = d[o + 2 * G * G:o + 2 * G * G + m["n_legendre"] * G * G].reshape(m["n_legendre"], G, G)
            for l in range(m["n_legendre"]):
                e[f"P{l + 1}"] = mom[l].tolist()
            mats.append(e)
        surfs = []
        for sf in self.surfaces:
            e = {"type": sf["kind"]}
            e.update({k: v for k, v in zip(keys[sf["kind"]], sf["c"])})
            e["boundary"] = sf["bc"]
            e["id"] = sf["id"]
            surfs.append(e)
        cells = []
        for c in self.cells:
            e = {"region": c["region"]}
            if c["material"] is not None:
                e["material"] = c["material"]
            else:
                e["universe"] = c["universe"]
            e["id"] = c["id"]
            cells.append(e)
        univs = []
        for uid in self.universe_decl:
            u = self.universes[uid]
            if u["kind"] == "cells":
                univs.append({"cells": u["cells"], "id": uid})
            else:
                e = {"id": uid, "type": "rectlinear", "shape": u["shape"], "pitch": u["pitch"],
                     "origin": u["origin"], "universes": u["tiles"]}
                if u["outer"] != -1:
                    e["outer"] = u["outer"]
                univs.append(e)
        srcs = []
        for so in self.sources:
            sp = ({"type": "point", "position": [so.low[a] for a in range(3)]} if so.spatial == abi.SPATIAL["point"]
                  else {"type": "box", "low": [so.low[a] for a in range(3)], "hi": [so.hi[a] for a in range(3)]})
            dr = ({"type": "isotropic"} if so.direction == abi.DIRECTION["isotropic"]
                  else {"type": "mono-directional", "direction": [so.dir[a] for a in range(3)]})
            src = {"spatial": sp, "direction": dr, "energy": {"type": "mono-energetic", "energy": so.energy_value},
                   "weight": so.weight}
            if so.fissile_only:  # a key of the source entry (src/source.cpp:104-110)
                src["fissile-only"] = True
            srcs.append(src)
        est = {v: k for k, v in abi.EST.items()}
        qty = {v: k for k, v in abi.QUANTITY.items()}
        # every mesh tally needs a unique name (src/collision_mesh_tally.cpp:210-230)
        tallies = [{"name": f"tally{i}", "shape": t["shape"], "low": t["low"], "hi": t["hi"],
                    "estimator": est[t["est"]], "quantity": qty[t["q"]],
                    "energy-bounds": np.asarray(t["eb"]).tolist()} for i, t in enumerate(self.tallies)]
        settings = {"nparticles": int(self.nparticles), "ngroups": G, "transport": self.tracking,
                    "simulation": self.mode, "energy-mode": "multi-group",
                    "energy-bounds": self.energy_bounds.tolist(), "seed": int(self.seed), "stride": int(self.stride)}
        settings["wgt-cutoff"] = float(self.wgt_cutoff)
        settings["wgt-survival"] = float(self.wgt_survival)
        settings["wgt-split"] = float(self.wgt_split)
        if self.mode == "branchless-k-eigenvalue":
            settings["branchless-material"] = self.branchless_material
            settings["branchless-splitting"] = self.branchless_splitting
            settings["branchless-combing"] = self.branchless_combing
        if ngenerations is not None:
            settings["ngenerations"] = int(ngenerations)
        if nignored is not None:
            settings["nignored"] = int(nignored)
        deck = {"materials": mats, "surfaces": surfs, "cells": cells, "universes": univs,
                "root-universe": self.root, "sources": srcs}
        if tallies:
            deck["tallies"] = tallies
        if self.entropy:
            deck["entropy"] = dict(self.entropy)
        if self.sampling_xs_ratio is not None:
            deck["sampling-xs-ratio"] = list(self.sampling_xs_ratio)  # a top-level key (src/parser.cpp:425-434)
        deck["settings"] = settings
        return deck

    # ------------------------------------------------------------- flattening
    def universe_order(self):
        """geometry::universes order of the reference parser."""
        order, made = [], set()
        cell_by_id = {c["id"]: c for c in self.cells}

        def make(uid):
            if uid in made:
                return
            if uid not in self.universes:
                raise ValueError(f"unknown universe id {uid}")
            u = self.universes[uid]
            if u["kind"] == "lattice":
                for t in u["tiles"]:
                    if t != -1:
                        make(t)
                if u["outer"] != -1:
                    make(u["outer"])
            else:
                for cid in u["cells"]:
                    if cid not in cell_by_id:
                        raise ValueError(f"universe {uid} references unknown cell {cid}")
            made.add(uid)
            order.append(uid)

        for c in self.cells:
            if c["universe"] is not None:
                make(c["universe"])
        for uid in self.universe_decl:
            make(uid)
        return order

    def build(self, precision=None, tracking=None):
        G = self.G
        surf_index = {s["id"]: i for i, s in enumerate(self.surfaces)}
        surf = (abi.Surface * max(1, len(self.surfaces)))()
        for i, s in enumerate(self.surfaces):
            surf[i].type = abi.SURF[s["kind"]]
            surf[i].bc = abi.BC[s["bc"]]
            surf[i].id = s["id"]
            for k, v in enumerate(s["c"]):
                surf[i].c[k] = v
        mat_index = {m["id"]: i for i, m in enumerate(self.materials)}
        order = self.universe_order()
        uni_index = {uid: i for i, uid in enumerate(order)}
        cell_index = {c["id"]: i for i, c in enumerate(self.cells)}
        rpn_all, cells = [], (abi.Cell * len(self.cells))()
        for i, c in enumerate(self.cells):
            rpn = infix_to_rpn(tokenize_region(c["region"], surf_index))
            cells[i].id = c["id"]
            cells[i].rpn_offset = len(rpn_all)
            cells[i].rpn_len = len(rpn)
            rpn_all += rpn
            if c["material"] is not None:
                cells[i].fill_kind = abi.FILL_MATERIAL
                cells[i].fill = mat_index[c["material"]]
            else:
                cells[i].fill_kind = abi.FILL_UNIVERSE
                cells[i].fill = uni_index[c["universe"]]
        cell_lists, lat_elems = [], []
        unis = (abi.Universe * len(order))()
        for i, uid in enumerate(order):
            u = self.universes[uid]
            unis[i].id = uid
            if u["kind"] == "cells":
                unis[i].kind = abi.UNIV_CELLS
                unis[i].list_offset = len(cell_lists)
                unis[i].list_len = len(u["cells"])
                cell_lists += [cell_index[cid] for cid in u["cells"]]
                unis[i].outer = -1
            else:
                unis[i].kind = abi.UNIV_RECT_LATTICE
                unis[i].list_offset = len(lat_elems)
                unis[i].list_len = len(u["tiles"])
                lat_elems += [-1 if t == -1 else uni_index[t] for t in u["tiles"]]
                unis[i].outer = -1 if u["outer"] == -1 else uni_index[u["outer"]]
                for a in range(3):
                    unis[i].shape[a] = u["shape"][a]
                    unis[i].pitch[a] = u["pitch"][a]
                    unis[i].origin[a] = u["origin"][a]
        mats = (abi.Material * len(self.materials))()
        data = []
        off = 0
        for i, m in enumerate(self.materials):
            mats[i].id = m["id"]
            mats[i].data_offset = off
            mats[i].n_legendre = m["n_legendre"]
            mats[i].n_delayed = m["n_delayed"]
            data.append(m["data"])
            off += m["data"].size
        mg = np.concatenate(data) if data else np.zeros(1)
        tal = (abi.MeshTally * max(1, len(self.tallies)))()
        teb = []
        for i, t in enumerate(self.tallies):
            tal[i].estimator = t["est"]
            tal[i].quantity = t["q"]
            for a in range(3):
                tal[i].shape[a] = t["shape"][a]
                tal[i].low[a] = t["low"][a]
                tal[i].hi[a] = t["hi"][a]
            tal[i].ebounds_offset = len(teb)
            tal[i].n_ebounds = len(t["eb"])
            teb += list(t["eb"])
        src = (abi.Source * max(1, len(self.sources)))(*self.sources)

        eb = np.ascontiguousarray(self.energy_bounds, dtype=np.float64)
        rpn_a = np.asarray(rpn_all if rpn_all else [0], dtype=np.int32)
        cl_a = np.asarray(cell_lists if cell_lists else [0], dtype=np.int32)
        le_a = np.asarray(lat_elems if lat_elems else [0], dtype=np.int32)
        mg_a = np.ascontiguousarray(mg, dtype=np.float64)
        teb_a = np.asarray(teb if teb else [0.0], dtype=np.float64)

        p = abi.Problem()
        s = p.settings
        s.mode = abi.MODE[self.mode]
        s.tracking = abi.TRACKING[tracking or self.tracking]
        s.precision = abi.PRECISION[precision or self.precision]
        s.ngroups = G
        s.seed = self.seed
        s.stride = self.stride
        s.wgt_cutoff = self.wgt_cutoff
        s.wgt_survival = self.wgt_survival
        s.nparticles = float(self.nparticles)
        s.block_size = self.block_size
        s.wgt_split = self.wgt_split
        s.branchless = 0
        if self.mode == "branchless-k-eigenvalue":
            s.branchless = (abi.BRANCHLESS_ON | (abi.BRANCHLESS_MATERIAL if self.branchless_material else 0) |
                            (abi.BRANCHLESS_SPLITTING if self.branchless_splitting else 0) |
                            (abi.BRANCHLESS_COMBING if self.branchless_combing else 0))
            s.global_rng_skip = (self.global_rng_skip if self.global_rng_skip is not None
                                 else 6 * (len(self.cells) + len(self.materials)))
        p.energy_bounds = _ptr(eb, C.c_double)
        p.surfaces = C.cast(surf, C.POINTER(abi.Surface))
        p.n_surfaces = len(self.surfaces)
        p.cells = C.cast(cells, C.POINTER(abi.Cell))
        p.n_cells = len(self.cells)
        p.rpn = _ptr(rpn_a, C.c_int32)
        p.n_rpn = len(rpn_all)
        p.universes = C.cast(unis, C.POINTER(abi.Universe))
        p.n_universes = len(order)
        p.cell_lists = _ptr(cl_a, C.c_int32)
        p.n_cell_lists = len(cell_lists)
        p.lattice_elems = _ptr(le_a, C.c_int32)
        p.n_lattice_elems = len(lat_elems)
        if self.root is None:
            raise ValueError("no root universe")
        p.root_universe = uni_index[self.root]
        p.materials = C.cast(mats, C.POINTER(abi.Material))
        p.n_materials = len(self.materials)
        p.mg_data = _ptr(mg_a, C.c_double)
        p.n_mg_data = mg_a.size
        p.tallies = C.cast(tal, C.POINTER(abi.MeshTally))
        p.n_tallies = len(self.tallies)
        p.tally_ebounds = _ptr(teb_a, C.c_double)
        p.n_tally_ebounds = len(teb)
        if self.entropy:
            p.entropy.enabled = 1
            for a in range(3):
                p.entropy.shape[a] = self.entropy["shape"][a]
                p.entropy.low[a] = self.entropy["low"][a]
                p.entropy.hi[a] = self.entropy["hi"][a]
        p.sources = C.cast(src, C.POINTER(abi.Source))
        p.n_sources = len(self.sources)
        smp = None
        if self.sampling_xs_ratio is not None:
            smp = np.asarray(self.sampling_xs_ratio, dtype=np.float64)
            if smp.shape != (G,):
                raise ValueError("sampling_xs_ratio needs one entry per group")
            p.sampling_xs_ratio = _ptr(smp, C.c_double)
        keep = [surf, cells, unis, mats, tal, src, eb, rpn_a, cl_a, le_a, mg_a, teb_a, smp]
        meta = {"universe_order": order, "tally_shapes": [t["shape"] for t in self.tallies],
                "tally_ne": [len(t["eb"]) - 1 for t in self.tallies], "ngroups": G,
                "nparticles": self.nparticles, "mode": self.mode}
        return Built(p, keep, meta)
