"""Seeded inputs and calls of the reference-pinned cases (TEST
INFRASTRUCTURE ONLY).

Each case builds an oracle State from the build's seeded generators (small
grids), names the reference subroutine that runs on it -- by its source
file and dummy arguments -- and the oracle call that restates it.  The
generator (make_golden.py) runs the reference routine on the state's
module arrays through f90exec and records a digest of every array and the
module scalars afterwards; the test (tests/test_golden_reference.py) runs
the oracle on the same state and compares.
"""
import hashlib

import numpy as np

import cappgpu
from cappgpu import FIELD_NAMES

from helpers import diag_dominant_matrix, randomize, with_fluxes

IP = 4

# Params members that are module variables of the reference under another
# name, or that configure the build only (no module variable).
PARAM_ALIASES = {"periodic": "periodic_boundary"}
BUILD_ONLY_PARAMS = {"isol_p", "piso_solver", "top_plane", "pad_"}
FIELD_ALIASES = {"walldist": "walldistance"}
BC_FACES = ("lbw", "lbe", "lbs", "lbn", "lbb", "lbt")

SCHEMES = {
    "uds": {}, "cds": {"lcds": 1}, "cds4": {"lcds4": 1}, "luds": {"lluds": 1}, "quick": {"lquds": 1},
    "smart": {"flux_limiter": 1, "lsmart": 1}, "avl": {"flux_limiter": 1, "lavl": 1},
    "muscl": {"flux_limiter": 1, "lmuscl": 1}, "umist": {"flux_limiter": 1, "lumist": 1},
    "gamma": {"flux_limiter": 1, "lgamma": 1},
}
NO_SCHEME = dict(lcds=0, lcds4=0, lluds=0, lquds=0, flux_limiter=0, lsmart=0, lavl=0, lmuscl=0, lumist=0,
                 lgamma=0)


class Case:
    """files: reference sources to translate (with the routines they call);
    ref: (subroutine, [actual arguments: module array names or ints]), or a
    list of such calls made in turn;
    oracle: callable(st) running the oracle's restatement;
    stubs: routines called only on branches the case does not take."""

    def __init__(self, name, build, files, ref, oracle, stubs=(), setup=(), switches=None, snippets=()):
        self.name, self.build, self.files, self.ref, self.oracle = name, build, files, ref, oracle
        self.stubs = tuple(stubs)
        # (name, parts) wrapped as subroutines, each part a statement text
        # or a (file, first line, last line) range of the reference: the
        # include fragments and the time-loop body of main.f90, with the
        # locals main.f90 declares for them
        self.snippets = tuple(snippets)
        # (file, first line, last line) of reference statements run before
        # the case, and module switches of the configuration (input file)
        self.setup = tuple(setup)
        self.switches = dict(switches or {})


def small_case(kind):
    return {"cavity": lambda: cappgpu.cases.cavity(N=(8, 7, 9)),
            "skewed": lambda: cappgpu.cases.poisson(N=(10, 9, 8)),
            "channel": lambda: cappgpu.cases.channel(N=(8, 6, 8))}[kind]()


def state(O, kind):
    case = small_case(kind)
    st = O.State.from_case(case, geometry_orient=1)
    with_fluxes(case, st)
    return case, st


def solver_state(O, seed, symmetric):
    st = O.State(14, 13, 12)
    rng = np.random.default_rng(seed)
    diag_dominant_matrix(st, rng, symmetric=symmetric)
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt"], -0.3, 0.3)
    randomize(st, rng, ["p", "res", "u"])
    st.params.update(dict(alfa=0.92, sor=[1e-8] * 10, nsw=[300] * 10, ipr=3, jpr=3, kpr=3))
    return None, st


def assembly_state(O, kind, seed):
    case, st = state(O, kind)
    rng = np.random.default_rng(seed)
    randomize(st, rng, ["u", "v", "w", "p", "pp"])
    randomize(st, rng, ["gradu_x", "gradu_y", "gradu_z", "gradv_x", "gradv_y", "gradv_z",
                        "gradw_x", "gradw_y", "gradw_z", "gradp_x", "gradp_y", "gradp_z"])
    randomize(st, rng, ["f1", "f2", "f3"], -0.5, 0.5)
    randomize(st, rng, ["vis", "den", "apu", "apv", "apw"], 0.5, 1.5)
    randomize(st, rng, ["su", "sv", "sw", "ae", "aw", "an", "as", "at", "ab", "ap", "sp", "spv"])
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt", "he", "hw", "hn", "hs", "ht", "hb"])
    randomize(st, rng, ["uo", "vo", "wo", "uoo", "voo", "woo", "t"])
    return case, st


def dir_args(case, d):
    nj, nij = case.nj, case.ni * case.nj
    return [(nj, 1, nij, "ar1x", "ar1y", "ar1z", "fx", "ae", "aw", "f1"),
            (1, nij, nj, "ar2x", "ar2y", "ar2z", "fy", "an", "as", "f2"),
            (nij, nj, 1, "ar3x", "ar3y", "ar3z", "fz", "at", "ab", "f3")][d]


# --------------------------------------------------------------------- cases

SOLVERS = [  # (oracle name, reference file, reference subroutine, symmetric matrix)
    ("sipsol", "sipsol.f90", "sipsol", False),
    ("pcgsip", "pcg-sip.f90", "pcgsip", True),
    ("iccg", "iccg.f90", "iccg", True),
    ("cgstab", "cgstab.f90", "cgstab", False),
    ("cgstab_sip", "cgstab_sip.f90", "cgstab_sip", False),
    ("dpcg", "pcg-jacobi.f90", "diagonally_preconditioned_cg", True),
]


def all_cases():
    cases = []

    for oname, f, sub, sym in SOLVERS:
        for seed in (20, 21):
            def build(O, seed=seed, sym=sym):
                return solver_state(O, seed, sym)
            cases.append(Case(f"solve_{oname}_{seed}", build, [f], (sub, ["p", IP]),
                              lambda st, o=oname: st.solve(o, "p", IP)))

        # stopped by the sweep limit: the report prints the loop index nsw + 1
        def build_short(O, sym=sym):
            _, st = solver_state(O, 22, sym)
            st.params.nsw[IP - 1] = 3
            return None, st
        cases.append(Case(f"solve_{oname}_nsw3", build_short, [f], (sub, ["p", IP]),
                          lambda st, o=oname: st.solve(o, "p", IP)))

    for periodic, f in ((0, "update_values_at_ghostcells_nonperiodic.f90"), (1, "update_values_at_ghostcells.f90")):
        def build(O, periodic=periodic):
            case, st = state(O, "skewed")
            rng = np.random.default_rng(10 + periodic)
            randomize(st, rng, ["u", "v", "w", "te", "ed", "t", "vis"], 0.1, 1.0)
            for face in BC_FACES:
                st.bc(face)[:] = rng.integers(1, 5, st.bc(face).size)
            st.params.periodic = periodic
            st.params.update(dict(uin=0.3, vin=-0.2, win=0.1, tein=0.05, edin=0.7, tin=1.5))
            return case, st
        cases.append(Case(f"ghost_cells_periodic{periodic}", build, [f], ("update_values_at_ghostcells", []),
                          lambda st: st.update_values_at_ghostcells()))

    for kind in ("cavity", "skewed", "channel"):
        def build(O, kind=kind):
            case, st = state(O, kind)
            randomize(st, np.random.default_rng(2), ["u", "gradu_x", "gradu_y", "gradu_z"])
            return case, st
        cases.append(Case(f"grad_gauss_{kind}", build, ["GRAD_GAUSS.f90"],
                          ("grad_gauss", ["u", "gradu_x", "gradu_y", "gradu_z"]),
                          lambda st: st.grad_gauss("u", "gradu_x", "gradu_y", "gradu_z")))

    def build_bpres(O):
        case, st = state(O, "skewed")
        randomize(st, np.random.default_rng(6), ["p"])
        return case, st
    cases.append(Case("bpres_skewed", build_bpres, ["bpres.f90"], ("bpres", ["p"]), lambda st: st.bpres("p")))

    def build_cbc(O):
        case, st = state(O, "cavity")
        randomize(st, np.random.default_rng(8), ["u", "v", "w", "f1", "f2"])
        return case, st
    cases.append(Case("correct_boundary_conditions_cavity", build_cbc, ["correctBoundaryConditions.f90"],
                      ("correctboundaryconditions", []), lambda st: st.correct_boundary_conditions()))

    for scheme in SCHEMES:
        for d in range(3):
            def build(O, scheme=scheme, d=d):
                case, st = assembly_state(O, "skewed", 30 + d)
                flags = dict(NO_SCHEME)
                flags.update(SCHEMES[scheme])
                st.params.update(flags)
                st.params.gds[0] = 0.9
                return case, st
            cases.append(Case(f"fluxuvw_{scheme}_{'xyz'[d]}", build, ["fluxuvw-overrelaxed-correction.f90"],
                              ("fluxuvw", ("dir", d)), ("fluxuvw", d)))

    for ipc in (0, 1):
        for d in range(3):
            def build(O, d=d):
                return assembly_state(O, "skewed", 40 + d)
            cases.append(Case(f"piso_assemble_pressure_eq_ipc{ipc}_{'xyz'[d]}", build,
                              ["PISO_assemble_pressure_eq.f90"],
                              ("piso_assemble_pressure_eq", ("dir", d, ipc, ["be", "bn", "bt"][d])),
                              ("piso_assemble_pressure_eq", d, ipc, ["be", "bn", "bt"][d])))

    for d in range(3):
        def build(O, d=d):
            return assembly_state(O, "skewed", 50 + d)
        cases.append(Case(f"assemble_pressure_eq_{'xyz'[d]}", build, ["assemble_pressure_eq.f90"],
                          ("assemble_pressure_eq", ("dir", d)), ("assemble_pressure_eq", d)))

    for d in range(3):
        def build(O, d=d):
            return assembly_state(O, "skewed", 60 + d)
        cases.append(Case(f"fluxmass_{'xyz'[d]}", build, ["fluxmass2.f90"],
                          ("fluxmass", ("dir", d)), ("fluxmass", d)))

    for cn in (0, 1):
        def build(O, cn=cn):
            case, st = assembly_state(O, "skewed", 70)
            st.params.update(dict(bdf=1, btime=1.0, cn=cn, timestep=0.01))
            return case, st
        cases.append(Case(f"piso_gethbya_cn{cn}", build, ["PISO_getHbyA.f90", "GRAD_GAUSS.f90"],
                          ("piso_gethbya", []), lambda st: st.piso_gethbya(), stubs=["grad_lsq_qr"]))

    for dims, flags in (((9, 8, 7), "all"), ((9, 8, 7), "some"), ((5, 6, 5), "all")):
        def build(O, dims=dims, flags=flags):
            st = O.State(*dims)
            rng = np.random.default_rng(31)
            randomize(st, rng, ["u", "v", "w", "te", "ed", "vis", "t", "f1", "f2", "f3"])
            randomize(st, rng, ["den", "ar1x", "ar1y", "ar1z"], 0.5, 1.5)
            for face in BC_FACES:
                b = st.bc(face)
                b[:] = rng.choice([1, 2, 2, 4], size=b.size)
            on = dict(low=1, loe=1, los=1, lon=1, lob=1, lot=1)
            if flags == "some":
                on.update(los=0, lot=0)
            st.params.update(dict(lout=1, flowin=0.9, **on))
            return None, st
        cases.append(Case(f"outbc_{dims[0]}x{dims[1]}x{dims[2]}_{flags}", build, ["outbc.f90"], ("outbc", []),
                          lambda st: st.outbc()))

    calcuvw_files = ["calcuvw.f90", "GRAD_GAUSS.f90", "fluxuvw-overrelaxed-correction.f90", "sipsol.f90",
                     "cgstab_sip.f90", "calcstress.f90"]
    for kind in ("cavity", "channel"):
        def build(O, kind=kind):
            case, st = state(O, kind)
            st.update_values_at_ghostcells()
            if kind == "channel":
                st.params.update(dict(timestep=0.05))
            return case, st
        cases.append(Case(f"calcuvw_{kind}", build, calcuvw_files, ("calcuvw", []), lambda st: st.calcuvw(),
                          stubs=["grad_lsq_qr", "additional_algebraic_stress_terms"]))

    def build_calcuvw_cn(O):
        case, st = state(O, "channel")
        st.update_values_at_ghostcells()
        st.params.update(dict(timestep=0.05, bdf=0, cn=1))
        return case, st
    cases.append(Case("calcuvw_channel_crank_nicolson", build_calcuvw_cn, calcuvw_files, ("calcuvw", []),
                      lambda st: st.calcuvw(), stubs=["grad_lsq_qr", "additional_algebraic_stress_terms"]))

    def build_piso_npcor2(O):
        case, st = state(O, "channel")
        st.params.update(dict(timestep=0.05, npcor=2))
        st.update_values_at_ghostcells()
        st.calcuvw()
        return case, st
    cases.append(Case("piso_multiple_correction_channel_npcor2", build_piso_npcor2,
                      ["PISO_multiple_correction.f90", "PISO_getHbyA.f90", "PISO_assemble_pressure_eq.f90",
                       "GRAD_GAUSS.f90", "bpres.f90", "outbc.f90", "pcg-sip.f90"],
                      ("piso_multiple_correction", []), lambda st: st.piso_multiple_correction(),
                      stubs=["grad_lsq_qr"]))

    def build_piso(O):
        case, st = state(O, "channel")
        st.params.update(dict(timestep=0.05))
        st.update_values_at_ghostcells()
        st.calcuvw()
        return case, st
    cases.append(Case("piso_multiple_correction_channel", build_piso,
                      ["PISO_multiple_correction.f90", "PISO_getHbyA.f90", "PISO_assemble_pressure_eq.f90",
                       "GRAD_GAUSS.f90", "bpres.f90", "outbc.f90", "pcg-sip.f90"],
                      ("piso_multiple_correction", []), lambda st: st.piso_multiple_correction(),
                      stubs=["grad_lsq_qr"]))

    for npcor in (1, 2):
        def build(O, npcor=npcor):
            case, st = state(O, "cavity")
            # the p' solver calcp hard-codes (calcp-multiple_correction_SIMPLE.f90:22, isol = 5)
            st.params.update(dict(npcor=npcor, isol_p=cappgpu.SOLVER["cgstab_sip"]))
            st.update_values_at_ghostcells()
            st.calcuvw()
            return case, st
        cases.append(Case(f"calcp_cavity_npcor{npcor}", build,
                          ["calcp-multiple_correction_SIMPLE.f90", "fluxmass2.f90", "fluxmc.f90", "GRAD_GAUSS.f90",
                           "bpres.f90", "outbc.f90", "correctBoundaryConditions.f90", "cgstab_sip.f90",
                           "pcg-sip.f90", "sipsol.f90", "iccg.f90", "cgstab.f90"],
                          ("calcp", []), lambda st: st.calcp(), stubs=["grad_lsq_qr"]))

    def build_les(O):
        case, st = state(O, "channel")
        p = st.params
        p.lles = 1
        p.lcal[cappgpu.params.IVIS - 1] = 1
        p.urf[cappgpu.params.IVIS - 1] = 0.7
        rng = np.random.default_rng(21)
        st.set_field("vis", st.field("vis") * (1 + 0.1 * rng.random(st.field("vis").size)))
        return case, st
    cases.append(Case("les_strain_and_viscosity_channel", build_les, ["find_strain_rate.f90", "calc_vis_les.f90",
                                                                      "GRAD_GAUSS.f90"],
                      [("find_strain_rate", []), ("calc_vis_les", [])],
                      lambda st: (st.find_strain_rate(), st.calc_vis_les()), stubs=["grad_lsq_qr"]))

    # Menter's k-omega SST from a developed state of a small RANS channel
    sst_files = ["calcscm.f90", "GRAD_GAUSS.f90", "find_strain_rate.f90", "calculate_stuff_for_sst.f90",
                 "fluxscm-overrelaxed-correction.f90", "sipsol.f90"]
    sst_setup = [("init.f90", 229, 245)]             # the SST constants
    sst_switches = {"lturb": True, "levm": True}     # sst itself is a Params member
    sst_stubs = ["grad_lsq_qr", "calculate_stuff_for_earsm", "von_karman_lengthscale"]
    for ifi, fname in ((5, "te"), (6, "ed")):
        cases.append(Case(f"calcscm_{fname}_rans_channel", sst_state, sst_files,
                          ("calcscm", [fname, "grad" + fname, ifi]), lambda st, ifi=ifi: st.calcscm(ifi),
                          stubs=sst_stubs, setup=sst_setup, switches=sst_switches))
    cases.append(Case("modvis_rans_channel", sst_state, ["modvis.f90", "calculate_stuff_for_sst.f90"],
                      ("modvis", []), lambda st: st.modvis(), stubs=sst_stubs, setup=sst_setup,
                      switches=sst_switches))

    # main.f90's include fragments, with the locals main.f90:32-37 declares
    def build_courant(O, conumfix=1):
        case, st = assembly_state(O, "channel", 80)
        st.params.update(dict(ltransient=1, conumfix=conumfix, conumfixvalue=0.5, timestep=0.01))
        return case, st
    for conumfix in (0, 1):
        cases.append(Case(f"courant_number_conumfix{conumfix}", lambda O, c=conumfix: build_courant(O, c), [],
                          ("courantno", []), lambda st: st.courant(),
                          snippets=[("courantno", "integer :: i, j, k, inp\nreal(prec) :: suma, dt\n"
                                                  "include 'CourantNo.h'")]))
    cases.append(Case("continuity_errors_channel", build_courant, [], ("continuityerrors", []),
                      lambda st: st.continuity_errors(),
                      snippets=[("continuityerrors", "integer :: i, j, k, inp, idew, idns, idtb\n"
                                                     "include 'continuityErrors.h'")]))

    def build_cmf(O):
        case, st = state(O, "channel")
        rng = np.random.default_rng(5)
        st.set_field("apu", 0.01 + 0.01 * rng.random(st.field("apu").size))
        st.params.uin = 1.3
        st.params.gradpcmf = 0.2
        return case, st
    cases.append(Case("const_massflux_correction_channel", build_cmf, [("fieldManipulation.f90",
                                                                         ["volumeweightedaverage"])],
                      ("constmflux", []), lambda st: st.const_massflux_correction(),
                      setup=[("init.f90", 356, 356)],          # magUbar = UIN
                      snippets=[("constmflux", "real(prec) :: magubarstar, ruaw, gragpplus, flowdirection\n"
                                               "include 'const_massflux_correction.f90'")]))

    # one PISO time step as main.f90's time loop runs it (:140-157 time
    # levels, :169 Courant number, :185-205 the iteration, :252 the mass-flux
    # correction), one iteration per step.  Left out, as the oracle's
    # drivers leave them out: bcin, abort_mission (:162, :171), the
    # residual normalisation and exit test (:218-240), and the output
    # calls.  find_strain_rate runs before calc_vis_les, which reads the
    # strain (calc_vis_les.f90:64) the LES path never forms.
    step = ["integer :: i, j, k, inp",
            "real(prec) :: suma, dt, magubarstar, ruaw, gragpplus, flowdirection",
            ("main.f90", 140, 157), ("main.f90", 169, 169), ("main.f90", 185, 203),
            "if(lcal(ivis) .and. lles) call find_strain_rate",
            ("main.f90", 205, 205),
            "if (ltransient .and. const_mflux) then", ("main.f90", 252, 252), "endif"]
    step_files = ["calcuvw.f90", "GRAD_GAUSS.f90", "fluxuvw-overrelaxed-correction.f90", "sipsol.f90",
                  "cgstab_sip.f90", "calcstress.f90", "outbc.f90", "PISO_multiple_correction.f90",
                  "PISO_getHbyA.f90", "PISO_assemble_pressure_eq.f90", "bpres.f90", "pcg-sip.f90",
                  "find_strain_rate.f90", "calc_vis_les.f90", "modvis.f90", "calcscm.f90",
                  "calculate_stuff_for_sst.f90", "fluxscm-overrelaxed-correction.f90",
                  ("fieldManipulation.f90", ["volumeweightedaverage"])]
    step_stubs = ["grad_lsq_qr", "additional_algebraic_stress_terms", "calcp", "pimple_multiple_correction",
                  "calcsct", "calculate_stuff_for_earsm", "von_karman_lengthscale"]

    def build_les_channel(O):
        case, st = state(O, "channel")
        st.params.lles = 1
        st.params.lcal[cappgpu.params.IVIS - 1] = 1
        return case, st
    cases.append(Case("piso_steps_les_channel_2", build_les_channel,
                      ["update_values_at_ghostcells.f90"] + step_files, [("pisostep", []), ("pisostep", [])],
                      lambda st: st.piso_steps(2), stubs=step_stubs, setup=[("init.f90", 356, 356)],
                      switches={"piso": True}, snippets=[("pisostep", step)]))
    def build_channel32(O):
        case = cappgpu.cases.channel(N=(32, 32, 32))   # the channel configuration (LES, mass flux) at 32^3
        st = O.State.from_case(case)
        with_fluxes(case, st)
        return case, st
    cases.append(Case("piso_step_channel32", build_channel32,
                      ["update_values_at_ghostcells.f90"] + step_files, ("pisostep", []),
                      lambda st: st.piso_steps(1), stubs=step_stubs, setup=[("init.f90", 356, 356)],
                      switches={"piso": True}, snippets=[("pisostep", step)]))
    cases.append(Case("piso_step_sst_channel", sst_state,
                      ["update_values_at_ghostcells.f90"] + step_files, ("pisostep", []),
                      lambda st: st.piso_steps(1), stubs=step_stubs,
                      setup=[("init.f90", 229, 245), ("init.f90", 356, 356)],
                      switches={"piso": True, "lturb": True, "levm": True}, snippets=[("pisostep", step)]))

    # face areas and interpolation factors as init.f90:50-141 forms them (its
    # cross products taken as written: the library's orientation 0) with
    # intfac.f90 and find_intersection_point.f90
    geo = ["integer :: i, j, k, intc, inbc, inp, ins, inb, inbs, idew, idns, idtb",
           "real(prec) :: ednom, tenom, dxet, dxzd, dyet, dyzd, dzet, dzzd, perturb",
           ("init.f90", 50, 141)]
    for kind in ("cavity", "skewed", "channel"):
        cases.append(Case(f"geometry_{kind}", lambda O, kind=kind: state(O, kind),
                          ["intfac.f90", "find_intersection_point.f90"], ("geometry", []),
                          lambda st: st.geometry(0), snippets=[("geometry", geo)]))

    # SIMPLE outer iterations: the iteration body of main.f90 (:185-205), steady
    simple_files = [f for f in step_files if f not in ("PISO_multiple_correction.f90", "PISO_getHbyA.f90",
                                                       "PISO_assemble_pressure_eq.f90")]
    simple_files += ["calcp-multiple_correction_SIMPLE.f90", "fluxmass2.f90", "fluxmc.f90",
                     "correctBoundaryConditions.f90", "iccg.f90", "cgstab.f90"]

    def build_simple(O):
        case, st = state(O, "cavity")
        st.params.isol_p = cappgpu.SOLVER["cgstab_sip"]    # calcp's own choice, isol = 5
        return case, st
    def build_simple32(O):
        case = cappgpu.cases.cavity(N=32)       # the configuration's own size and parameters
        st = O.State.from_case(case, geometry_orient=1)
        with_fluxes(case, st)
        st.params.isol_p = cappgpu.SOLVER["cgstab_sip"]
        return case, st
    cases.append(Case("simple_iters_cavity32_2", build_simple32,
                      ["update_values_at_ghostcells_nonperiodic.f90"] + simple_files,
                      [("simpleiter", []), ("simpleiter", [])], lambda st: st.simple_iters(2),
                      stubs=[x for x in step_stubs if x != "calcp"] + ["piso_multiple_correction"],
                      switches={"simple": True},
                      snippets=[("simpleiter", [("main.f90", 185, 205)])]))
    def build_simple_outlet(O):
        case, st = state(O, "cavity")
        st.bc("lbw")[:] = 1
        st.bc("lbe")[:] = 2
        st.params.update(dict(uin=0.5, lout=1, loe=1, flowin=0.02, const_mflux=0,
                              isol_p=cappgpu.SOLVER["cgstab_sip"]))
        return case, st
    cases.append(Case("simple_iters_cavity_inflow_outflow_2", build_simple_outlet,
                      ["update_values_at_ghostcells_nonperiodic.f90"] + simple_files,
                      [("simpleiter", []), ("simpleiter", [])], lambda st: st.simple_iters(2),
                      stubs=[x for x in step_stubs if x != "calcp"] + ["piso_multiple_correction"],
                      switches={"simple": True},
                      snippets=[("simpleiter", [("main.f90", 185, 205)])]))
    cases.append(Case("simple_iters_cavity_2", build_simple,
                      ["update_values_at_ghostcells_nonperiodic.f90"] + simple_files,
                      [("simpleiter", []), ("simpleiter", [])], lambda st: st.simple_iters(2),
                      stubs=[x for x in step_stubs if x != "calcp"] + ["piso_multiple_correction"],
                      switches={"simple": True},
                      snippets=[("simpleiter", [("main.f90", 185, 205)])]))
    return cases


def sst_state(O):
    """A small RANS channel one PISO step (with the SST equations) old."""
    case = cappgpu.cases.rans_channel(N=(16, 12, 16))
    st = O.State.from_case(case)
    with_fluxes(case, st)
    st.piso_steps(1)
    return case, st


def reference_calls(case_obj, grid_case):
    """The reference subroutines the case runs, with their actual arguments."""
    calls = case_obj.ref if isinstance(case_obj.ref, list) else [case_obj.ref]
    out = []
    for sub, args in calls:
        if isinstance(args, tuple) and args[0] == "dir":
            out.append((sub, list(dir_args(grid_case, args[1])) + list(args[2:])))
        else:
            out.append((sub, list(args)))
    return out


def run_oracle(case_obj, grid_case, st):
    if callable(case_obj.oracle):
        return case_obj.oracle(st)
    name, d = case_obj.oracle[0], case_obj.oracle[1]
    a = dir_args(grid_case, d)
    return getattr(st, name)(*a, *case_obj.oracle[2:])


# ------------------------------------------------------------------ digests

def field_digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()[:24]


def all_fields_digest(digests):
    """One digest over the per-array digests of every module array."""
    return hashlib.sha256("".join(digests[n] for n in FIELD_NAMES).encode()).hexdigest()[:24]


def params_digest(params):
    return hashlib.sha256(repr(sorted(params.items())).encode()).hexdigest()[:24]


def state_digest(st):
    h = hashlib.sha256()
    for n in FIELD_NAMES:
        h.update(np.ascontiguousarray(st.field(n), dtype=np.float64).tobytes())
    for face in BC_FACES:
        h.update(np.ascontiguousarray(st.bc(face), dtype=np.int32).tobytes())
    for name, _ in type(st.params)._fields_:
        v = getattr(st.params, name)
        h.update(repr(list(v) if hasattr(v, "__len__") else v).encode())
    return h.hexdigest()[:32]


def params_record(values):
    """{name: value} of the module scalars compared after a call; floats as
    exact hex strings."""
    out = {}
    for k, v in values.items():
        if isinstance(v, (list, tuple)):
            out[k] = [float(x).hex() if isinstance(x, float) else int(x) for x in v]
        elif isinstance(v, float):
            out[k] = float(v).hex()
        else:
            out[k] = int(v)
    return out


def oracle_params(st):
    vals = {}
    for name, ctype in type(st.params)._fields_:
        if name in BUILD_ONLY_PARAMS:
            continue
        v = getattr(st.params, name)
        if hasattr(v, "__len__"):
            vals[name] = [float(x) if isinstance(x, float) else int(x) for x in v]
        else:
            vals[name] = float(v) if isinstance(v, float) else int(v)
    return params_record(vals)
