"""Run configurations of the mpcmd engine.

``mpcmd_config`` (include/mpcmd.h) carries the reference input decks after the
derivations the reference drivers make:

* ``read_collective_input`` / ``collective_config`` follow
  collective_code/main_pattern.f95:19-64 (44 positional values) and :66-127
  (particle numbers from the densities, MPCtstep, sphere masses);
* ``read_selkov_input`` / ``selkov_config`` follow
  selkov_code/Main_SelkovDimer.f90:7-45 and :47-105 (T = T/5, Vol = 64000
  hard-coded in Global_SelkovDimer.f90:30, rotang = pi/2 at :326);
* ``workload`` builds the synthetic benchmark workloads (seeded, no external
  data): c0 plain single dimer 30^3 periodic, c1 collective quasi-2D
  128x128x16 with walls and 64 dimers, c2 Selkov kinetics 256^3 with 512
  dimers, each optionally scaled down for tests.
"""
import ctypes as C
import math

_I32, _I64, _U64, _D = C.c_int32, C.c_int64, C.c_uint64, C.c_double

FIELDS = [
    ("lx", _I32), ("ly", _I32), ("lz", _I32), ("geometry", _I32), ("n_dimers", _I32),
    ("kinetics", _I32), ("exclusion", _I32), ("catalysis", _I32), ("rotation_sense", _I32),
    ("mpc_every", _I32), ("sort_every", _I32), ("react_box_type", _I32), ("react_dir", _I32),
    ("cell_capacity", _I32), ("max_neighbour", _I32), ("rattle_max_iter", _I32),
    ("init_plane", _I32), ("pad0", _I32),
    ("n_solvent", _I64), ("seed", _U64), ("init_count", _I64 * 4),
    ("mass", _D * 4), ("eps_c", _D * 4), ("eps_n", _D * 4),
    ("rc", _D), ("rn", _D), ("dcn", _D), ("mc", _D), ("mn", _D), ("rw", _D), ("ew", _D),
    ("rm_delta", _D), ("em", _D), ("rp_ab", _D), ("rp_ba", _D), ("kT", _D), ("skin", _D),
    ("rot_angle", _D), ("md_dt", _D), ("mpc_dt", _D), ("k", _D * 6),
    ("precision", _I32), ("shell_capacity", _I32),
    ("variant", _I32), ("layout", _I32), ("layout_rows", _I32), ("layout_cols", _I32),
    ("owner_tags", _I32), ("reserved", _I32), ("tether_k", _D), ("tether_z", _D), ("layout_sep", _D),
]

GEOM_WALLS, GEOM_PERIODIC = 0, 1
KIN_NONE, KIN_SIMPLE, KIN_SELKOV = 0, 1, 2
EXCL_PARTICLE, EXCL_CELLS = 0, 1
CAT_DETERMINISTIC, CAT_PROBABILISTIC, CAT_ON_EXIT = 0, 1, 2
PREC_FP32, PREC_FP64 = 32, 64
VARIANT_MOTOR, VARIANT_ROTOR = 0, 1
LAYOUT_RANDOM, LAYOUT_GRID, LAYOUT_LINE = 0, 1, 2


class MpcmdConfig(C.Structure):
    _fields_ = FIELDS


def to_struct(cfg):
    s = MpcmdConfig()
    for name, typ in FIELDS:
        if name not in cfg:
            continue
        v = cfg[name]
        if hasattr(typ, "_length_"):
            arr = getattr(s, name)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(s, name, v)
    return s


def sphere_masses(n_solvent, ncell, rc, rn):
    """main_pattern.f95:118-119: density-matched sphere masses."""
    rho = n_solvent / float(ncell)
    return rho * ((4.0 * math.pi) / 3) * rc ** 3, rho * ((4.0 * math.pi) / 3) * rn ** 3


def base_config(**kw):
    """Defaults of the collective input deck (collective_code/input.txt)."""
    cfg = dict(
        lx=16, ly=16, lz=16, geometry=GEOM_PERIODIC, n_dimers=1, kinetics=KIN_SIMPLE,
        exclusion=EXCL_PARTICLE, catalysis=CAT_DETERMINISTIC, rotation_sense=1,
        mpc_every=50, sort_every=10000, react_box_type=6, react_dir=0, cell_capacity=100,
        max_neighbour=30000, rattle_max_iter=100000, init_plane=0, pad0=0,
        n_solvent=0, seed=1, init_count=[0, 0, 0, 0],
        mass=[1.0, 1.0, 1.0, 1.0], eps_c=[1.0, 1.0, 1.0, 1.0], eps_n=[1.0, 0.1, 1.0, 1.0],
        rc=4.0, rn=2.0, dcn=6.5, mc=0.0, mn=0.0, rw=1.0, ew=1.0, rm_delta=1.0, em=1.0,
        rp_ab=1.0, rp_ba=0.0, kT=1.0 / 6.0, skin=1.5, rot_angle=2.0 * math.pi / 3.0,
        md_dt=0.01, mpc_dt=0.5, k=[0.01, 0, 0, 0, 0, 0],
        precision=PREC_FP32, shell_capacity=0, variant=VARIANT_MOTOR, layout=LAYOUT_RANDOM, layout_rows=0,
        layout_cols=0, owner_tags=0, reserved=0, tether_k=0.0, tether_z=0.0, layout_sep=0.0,
    )
    cfg.update(kw)
    return finish(cfg)


def finish(cfg, density=10.0):
    """Fill the derived fields (particle count, species counts, masses)."""
    ncell = cfg["lx"] * cfg["ly"] * cfg["lz"]
    if not cfg.get("n_solvent"):
        cfg["n_solvent"] = int(round(density * ncell))
    if sum(cfg["init_count"]) != cfg["n_solvent"]:
        cfg["init_count"] = [cfg["n_solvent"], 0, 0, 0]
    if not cfg.get("mc") or not cfg.get("mn"):
        cfg["mc"], cfg["mn"] = sphere_masses(cfg["n_solvent"], ncell, cfg["rc"], cfg["rn"])
    cfg["mpc_every"] = int(round(cfg["mpc_dt"] / cfg["md_dt"]))
    return cfg


# ------------------------------------------------------------ reference decks --
COLLECTIVE_KEYS = [
    "ini_seed", "tstep", "rhoa", "rhob", "rhos", "box1", "box2", "box3", "numdims", "Ma", "Mb", "Ms",
    "Rc", "Rn", "Dcn", "EaC", "EbC", "EsC", "EaN", "EbN", "EsN", "Rw", "Ew", "Rm_delta", "Em",
    "RPab", "RPba", "T", "skinrad", "a0", "rotang", "MDt", "MPCt", "sort_step", "k1",
    "x_conc_slab", "y_conc_slab", "z_conc_slab", "react_box_type", "react_dir",
    "Freq1", "Freq2", "Freq3", "Freq4",
]
SELKOV_KEYS = [
    "seed", "Nf0", "Ng0", "Ni0", "box1", "box2", "box3", "Mf", "Mg", "Mi", "Rc", "Rn", "Dcn",
    "EfC", "EgC", "EiC", "EfN", "EgN", "EiN", "RPfg", "RPgf", "T", "A0", "MDt", "MPCt",
    "k1", "k2", "k3", "k4", "k5", "k6", "Freq1", "Freq2", "Freq3", "Freq4", "Freq5", "Freq6",
]

# rotational_code/2d_array/main_rotation.f95:17-51 and
# rotational_code/linear_periodic_ci/main_rotation.f95:17-49
ROTATIONAL_GRID_KEYS = [
    "seed", "tstep", "rhoa", "rhob", "box1", "box2", "box3", "sep", "numrows", "numcols", "Ma", "Mb",
    "Rc", "Rn", "Dcn", "EaC", "EbC", "EaN", "EbN", "k_harm", "gap", "RPab", "RPba", "T", "skinrad",
    "a0", "rotang", "MDt", "MPCt", "sort_step", "k1", "Freq1", "Freq2", "Freq3", "Freq4",
]
ROTATIONAL_LINE_KEYS = [
    "seed", "tstep", "rhoa", "rhob", "box1", "box2", "box3", "numdims", "Ma", "Mb",
    "Rc", "Rn", "Dcn", "EaC", "EbC", "EaN", "EbN", "k_harm", "gap", "RPab", "RPba", "T", "skinrad",
    "a0", "rotang", "MDt", "MPCt", "sort_step", "k1", "Freq1", "Freq2", "Freq3", "Freq4",
]


def _fortran_number(tok):
    t = tok.strip().lower().replace("d", "e")
    if t.endswith("."):
        t = t[:-1]
    return float(t)


def read_deck(path, keys):
    """Positional free-format deck: the first token of each line is the value."""
    vals = []
    with open(path) as f:
        for line in f:
            if line.strip():
                vals.append(_fortran_number(line.split()[0]))
    if len(vals) < len(keys):
        raise ValueError("%s: %d values, expected %d" % (path, len(vals), len(keys)))
    return dict(zip(keys, vals[: len(keys)]))


def read_collective_input(path):
    return read_deck(path, COLLECTIVE_KEYS)


def read_selkov_input(path):
    return read_deck(path, SELKOV_KEYS)


def collective_config(deck, **kw):
    """main_pattern.f95:66-127."""
    box = [int(deck["box1"]), int(deck["box2"]), int(deck["box3"])]
    vol = box[0] * box[1] * box[2]
    nd = int(deck["numdims"])
    vact = vol - nd * ((4.0 * math.pi * deck["Rc"] ** 3) / 3.0 + (4.0 * math.pi * deck["Rn"] ** 3) / 3.0)
    na0 = math.floor(deck["rhoa"] * vact)
    nb0 = math.floor(deck["rhob"] * vact)
    ns0 = math.floor(deck["rhob"] * vact)   # main_pattern.f95:70 uses rhob for S
    nt = na0 + nb0 + ns0
    mc, mn = sphere_masses(nt, vol, deck["Rc"], deck["Rn"])
    cfg = dict(
        lx=box[0], ly=box[1], lz=box[2], geometry=GEOM_WALLS, n_dimers=nd, kinetics=KIN_SIMPLE,
        exclusion=EXCL_PARTICLE, catalysis=CAT_DETERMINISTIC, rotation_sense=1,
        mpc_every=int(deck["MPCt"] / deck["MDt"]), sort_every=int(deck["sort_step"]),
        react_box_type=int(deck["react_box_type"]), react_dir=int(deck["react_dir"]),
        cell_capacity=100, max_neighbour=30000, rattle_max_iter=100000, init_plane=0, pad0=0,
        n_solvent=nt, seed=int(deck["ini_seed"]), init_count=[na0, nb0, ns0, 0],
        mass=[deck["Ma"], deck["Mb"], deck["Ms"], 1.0],
        eps_c=[deck["EaC"], deck["EbC"], deck["EsC"], 0.0], eps_n=[deck["EaN"], deck["EbN"], deck["EsN"], 0.0],
        rc=deck["Rc"], rn=deck["Rn"], dcn=deck["Dcn"], mc=mc, mn=mn, rw=deck["Rw"], ew=deck["Ew"],
        rm_delta=deck["Rm_delta"], em=deck["Em"], rp_ab=deck["RPab"], rp_ba=deck["RPba"], kT=deck["T"],
        skin=deck["skinrad"], rot_angle=deck["rotang"], md_dt=deck["MDt"], mpc_dt=deck["MPCt"],
        k=[deck["k1"], 0, 0, 0, 0, 0], precision=PREC_FP32, shell_capacity=0, reserved=0,
    )
    cfg.update(kw)
    return cfg


def read_rotational_input(path, layout=LAYOUT_GRID):
    return read_deck(path, ROTATIONAL_GRID_KEYS if layout == LAYOUT_GRID else ROTATIONAL_LINE_KEYS)


def rotational_config(deck, layout=LAYOUT_GRID, **kw):
    """rotational_code/2d_array/main_rotation.f95:53-110 (grid of rotors) or
    linear_periodic_ci/main_rotation.f95:51-108 (line of rotors, sep derived
    at :52): anchored dimers with a harmonic z tether over a walled box, no
    motor-motor LJ, no reactive floor, reaction_simple with the rate k1.
    ``owner_tags=1`` gives linear_periodic_no_ci (type_B owner tags)."""
    box = [int(deck["box1"]), int(deck["box2"]), int(deck["box3"])]
    vol = box[0] * box[1] * box[2]
    cutoff = 2.0 ** (1.0 / 6.0)
    if layout == LAYOUT_GRID:
        rows, cols = int(deck["numrows"]), int(deck["numcols"])
        nd = rows * cols
        sep = deck["sep"]
    else:
        rows, cols = 0, 0
        nd = int(deck["numdims"])
        sep = (deck["box1"] - nd * (2.0 * deck["Rc"] * cutoff + deck["Dcn"])) / nd
    # Vact as the drivers compute it (the N-sphere volume enters with a minus)
    vact = vol - nd * ((4.0 * math.pi * deck["Rc"] ** 3) / 3.0 - (4.0 * math.pi * deck["Rn"] ** 3) / 3.0)
    na0 = math.floor(deck["rhoa"] * vact)
    nb0 = math.floor(deck["rhob"] * vact)
    nt = na0 + nb0
    mc, mn = sphere_masses(nt, vol, deck["Rc"], deck["Rn"])
    cfg = dict(
        lx=box[0], ly=box[1], lz=box[2], geometry=GEOM_WALLS, n_dimers=nd, kinetics=KIN_SIMPLE,
        exclusion=EXCL_PARTICLE, catalysis=CAT_DETERMINISTIC, rotation_sense=1,
        mpc_every=int(round(deck["MPCt"] / deck["MDt"])), sort_every=int(deck["sort_step"]),
        react_box_type=0, react_dir=0, cell_capacity=100, max_neighbour=30000, rattle_max_iter=100000,
        init_plane=0, pad0=0, n_solvent=nt, seed=int(deck["seed"]), init_count=[na0, nb0, 0, 0],
        mass=[deck["Ma"], deck["Mb"], 1.0, 1.0], eps_c=[deck["EaC"], deck["EbC"], 0.0, 0.0],
        eps_n=[deck["EaN"], deck["EbN"], 0.0, 0.0], rc=deck["Rc"], rn=deck["Rn"], dcn=deck["Dcn"],
        mc=mc, mn=mn, rw=1.0, ew=0.0, rm_delta=0.0, em=0.0, rp_ab=deck["RPab"], rp_ba=deck["RPba"],
        kT=deck["T"], skin=deck["skinrad"], rot_angle=deck["rotang"], md_dt=deck["MDt"], mpc_dt=deck["MPCt"],
        k=[deck["k1"], 0, 0, 0, 0, 0], precision=PREC_FP32, shell_capacity=0,
        variant=VARIANT_ROTOR, layout=layout, layout_rows=rows, layout_cols=cols, owner_tags=0, reserved=0,
        tether_k=deck["k_harm"], tether_z=deck["Rc"] + deck["gap"], layout_sep=sep,
    )
    cfg.update(kw)
    return cfg


def selkov_config(deck, **kw):
    """Main_SelkovDimer.f90:47-105 (single dimer, fully periodic)."""
    box = [int(deck["box1"]), int(deck["box2"]), int(deck["box3"])]
    nt = int(deck["Nf0"] + deck["Ng0"] + deck["Ni0"])
    vol = 64000  # Global_SelkovDimer.f90:30
    mc, mn = sphere_masses(nt, vol, deck["Rc"], deck["Rn"])
    cfg = dict(
        lx=box[0], ly=box[1], lz=box[2], geometry=GEOM_PERIODIC, n_dimers=1, kinetics=KIN_SELKOV,
        exclusion=EXCL_CELLS, catalysis=CAT_PROBABILISTIC, rotation_sense=-1,
        mpc_every=int(deck["MPCt"] / deck["MDt"]), sort_every=10000, react_box_type=7, react_dir=0,
        cell_capacity=200, max_neighbour=30000, rattle_max_iter=100000, init_plane=0, pad0=0,
        n_solvent=nt, seed=int(deck["seed"]), init_count=[int(deck["Nf0"]), int(deck["Ng0"]), 0, int(deck["Ni0"])],
        mass=[deck["Mf"], deck["Mg"], 1.0, deck["Mi"]],
        eps_c=[deck["EfC"], deck["EgC"], 0.0, deck["EiC"]], eps_n=[deck["EfN"], deck["EgN"], 0.0, deck["EiN"]],
        rc=deck["Rc"], rn=deck["Rn"], dcn=deck["Dcn"], mc=mc, mn=mn, rw=1.0, ew=1.0, rm_delta=1.0, em=1.0,
        rp_ab=deck["RPfg"], rp_ba=deck["RPgf"], kT=deck["T"] / 5.0, skin=1.5, rot_angle=math.pi / 2,
        md_dt=deck["MDt"], mpc_dt=deck["MPCt"],
        k=[deck["k1"], deck["k2"], deck["k3"], deck["k4"], deck["k5"], deck["k6"]],
        precision=PREC_FP32, shell_capacity=0, reserved=0,
    )
    cfg.update(kw)
    return cfg


# ----------------------------------------------------------------- workloads --
SELKOV_FRACTIONS = (230400, 54400, 422400)   # F : G : I of the Selkov input deck


def workload(name, scale=1.0, **kw):
    """Synthetic benchmark workloads.  ``scale`` shrinks the box edges (and the
    dimer count with the volume) for tests; scale=1 is the full size."""
    name = name.lower()
    if name == "c0":
        L = max(8, int(round(30 * scale)))
        args = dict(lx=L, ly=L, lz=L, geometry=GEOM_PERIODIC, n_dimers=1)
    elif name == "c1":
        lx = max(8, int(round(128 * scale)))
        nd = max(1, int(round(64 * scale * scale)))
        args = dict(lx=lx, ly=lx, lz=16, geometry=GEOM_WALLS, n_dimers=nd, init_plane=1)
    elif name == "c2":
        L = max(8, int(round(256 * scale)))
        nd = max(1, int(round(512 * scale ** 3)))
        n = 10 * L ** 3
        tot = sum(SELKOV_FRACTIONS)
        nf = n * SELKOV_FRACTIONS[0] // tot
        ng = n * SELKOV_FRACTIONS[1] // tot
        args = dict(lx=L, ly=L, lz=L, geometry=GEOM_PERIODIC, n_dimers=nd, kinetics=KIN_SELKOV,
                    exclusion=EXCL_CELLS, catalysis=CAT_PROBABILISTIC, rotation_sense=-1,
                    cell_capacity=200, n_solvent=n, init_count=[nf, ng, 0, n - nf - ng],
                    eps_c=[1.0, 1.0, 0.0, 1.0], eps_n=[1.0, 0.1, 0.0, 1.0],
                    k=[1.0, 0.1, 1.0, 0.0, 0.01, 0.0], sort_every=10000)
    elif name in ("rot", "rot_line", "rot_owner"):
        # rotors of rotational_code/2d_array (a grid) or linear_periodic_ci (a
        # line) with their input decks' parameters, scaled with the box
        lx = max(16, int(round((64 if name == "rot" else 256) * scale)))
        ly = max(16, int(round(64 * scale)))
        lz = max(8, int(round(32 * scale)))
        rc = rn = 2.0
        dcn = 5.0
        pitch = dcn + 2.0 * rc * 2.0 ** (1.0 / 6.0)
        common = dict(lx=lx, ly=ly, lz=lz, geometry=GEOM_WALLS, kinetics=KIN_SIMPLE, react_box_type=0,
                      rc=rc, rn=rn, dcn=dcn, eps_c=[0.1, 0.1, 0.0, 0.0] if name == "rot" else [1.0, 1.0, 0.0, 0.0],
                      eps_n=[0.1, 1.0, 0.0, 0.0], rw=1.0, ew=0.0, rm_delta=0.0, em=0.0, kT=0.2, skin=0.7,
                      rot_angle=math.pi / 2, md_dt=0.005, mpc_dt=0.1, k=[0.001, 0, 0, 0, 0, 0],
                      variant=VARIANT_ROTOR, tether_k=1000.0, tether_z=rc + 1.0)
        if name == "rot":
            n = max(1, min(6, int(lx // pitch), int(ly // pitch)))
            args = dict(common, n_dimers=n * n, layout=LAYOUT_GRID, layout_rows=n, layout_cols=n, layout_sep=0.0)
        else:
            # rot_owner: the line of linear_periodic_no_ci, B particles tagged
            # with the motor that made them
            nd = max(1, int(lx // pitch) // 2)
            args = dict(common, n_dimers=nd, layout=LAYOUT_LINE, layout_sep=(lx - nd * pitch) / nd,
                        owner_tags=1 if name == "rot_owner" else 0)
    else:
        raise ValueError("unknown workload %r" % name)
    if "n_solvent" in kw and "init_count" not in kw and name == "c2":
        n = kw["n_solvent"]
        tot = sum(SELKOV_FRACTIONS)
        nf = n * SELKOV_FRACTIONS[0] // tot
        ng = n * SELKOV_FRACTIONS[1] // tot
        args["init_count"] = [nf, ng, 0, n - nf - ng]
    args.update(kw)
    return base_config(**args)


WORKLOAD_STEPS = {"c0": 100, "c1": 1000, "c2": 200}   # MPC steps of each workload
