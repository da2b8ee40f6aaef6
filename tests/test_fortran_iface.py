"""The Fortran iso_c_binding shim (fortran/cappgpu_iface.f90) against the C
header it binds.

No Fortran compiler exists where this library is built or tested, so the
shim is checked by reading it: every bind(c) interface names a function
that include/cappgpu.h declares, with the same number of arguments passed
the same way (by value or by address, of the same C type); the field ids,
solver codes and the two bind(c) derived types match the header's; every
drop-in keeps the name and dummy arguments of the reference subroutine it
replaces; and every reference file the shim's header comment says it
replaces has its drop-in.  (No GPU work here.)"""
import re

import pytest

from conftest import ROOT

SHIM = ROOT / "cappuccino-ghostcells-mpi_gb300" / "fortran" / "cappgpu_iface.f90"
HEADER = ROOT / "include" / "cappgpu.h"

# reference subroutine statements the drop-ins reproduce (name, dummies)
REFERENCE_DROPINS = {
    "pcg-sip.f90": ("pcgsip", ["fi", "ifi"]),                                   # pcg-sip.f90:3
    "sipsol.f90": ("sipsol", ["fi", "ifi"]),                                    # sipsol.f90:3
    "iccg.f90": ("iccg", ["fi", "ifi"]),                                        # iccg.f90:3
    "cgstab.f90": ("cgstab", ["fi", "ifi"]),                                    # cgstab.f90:1
    "cgstab_sip.f90": ("cgstab_sip", ["fi", "ifi"]),                            # cgstab_sip.f90:1
    "pcg-jacobi.f90": ("diagonally_preconditioned_cg", ["fi", "ifi"]),          # pcg-jacobi.f90:3
    "GRAD_GAUSS.f90": ("grad_gauss", ["u", "dudx", "dudy", "dudz"]),             # GRAD_GAUSS.f90:1
    "fluxuvw-overrelaxed-correction.f90": (
        "fluxuvw", ["idew", "idns", "idtb", "arvx", "arvy", "arvz", "fif", "acfe", "acfw", "fcf"]),  # :3-5
    "calcuvw.f90": ("calcuvw", []),                                             # calcuvw.f90:3
    "PISO_assemble_pressure_eq.f90": (
        "piso_assemble_pressure_eq",
        ["idew", "idns", "idtb", "arvx", "arvy", "arvz", "fif", "acfe", "acfw", "fcf", "ipc", "bp"]),  # :3-5
    "assemble_pressure_eq.f90": (
        "assemble_pressure_eq", ["idew", "idns", "idtb", "arvx", "arvy", "arvz", "fif", "acfe", "acfw", "fcf"]),
    "PISO_getHbyA.f90": ("piso_gethbya", []),                                   # PISO_getHbyA.f90:3
    "PISO_multiple_correction.f90": ("piso_multiple_correction", []),           # PISO_multiple_correction.f90:3
    "bpres.f90": ("bpres", ["p"]),                                              # bpres.f90:3
    "update_values_at_ghostcells*.f90": ("update_values_at_ghostcells", []),    # both forms, :3
    "calcscm.f90": ("calcscm", ["fi", "gradfi", "ifi"]),                        # calcscm.f90:3
    "modvis.f90": ("modvis", []),                                               # modvis.f90:3
    "exchange_mpi.f90": ("exchange", ["phi"]),                                  # exchange_mpi.f90:4
    "global_sum_mpi.f90": ("global_sum", ["phi"]),                              # global_sum_mpi.f90:4
    "global_max_mpi.f90": ("global_max", ["phi"]),                              # global_max_mpi.f90:4
}


def fortran_statements(text):
    """Fortran free-form source as statements: comments dropped,
    continuation lines joined, lower case."""
    out, cur = [], ""
    for line in text.splitlines():
        line = re.sub(r"!.*", "", line) if "'" not in line and '"' not in line else _strip_comment(line)
        line = line.rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if cur:
            s = s[1:] if s.startswith("&") else s
            cur += " " + s
        else:
            cur = s
        if cur.endswith("&"):
            cur = cur[:-1]
            continue
        out.append(re.sub(r"\s+", " ", cur).lower())
        cur = ""
    return out


def _strip_comment(line):
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i]
    return line


def c_text():
    return re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)


def c_prototypes():
    """name -> list of C parameter type strings (names dropped)."""
    protos = {}
    for m in re.finditer(r"\bint\s+(cappgpu_\w+)\s*\(([^)]*)\)\s*;", c_text()):
        args = [a.strip() for a in m.group(2).split(",")]
        if args == ["void"]:
            args = []
        types = []
        for a in args:
            a = re.sub(r"\s+", " ", a)
            mm = re.match(r"(.*?)(\w+)$", a)
            types.append(mm.group(1).replace(" *", "*").strip())
        protos[m.group(1)] = types
    return protos


def c_enum_values(enum_name):
    body = re.search(r"enum\s+%s\s*\{(.*?)\}" % enum_name, c_text(), flags=re.S).group(1)
    vals, nxt = {}, 0
    for item in body.split(","):
        item = item.strip()
        if not item:
            continue
        if "=" in item:
            name, v = (s.strip() for s in item.split("="))
            nxt = int(v)
        else:
            name = item
        vals[name] = nxt
        nxt += 1
    return vals


def c_defines(prefix):
    return {m.group(1): int(m.group(2))
            for m in re.finditer(r"#define\s+(%s\w*)\s+(-?\d+)" % prefix, HEADER.read_text())}


def c_struct_members(name):
    text = c_text()
    body = re.search(r"typedef struct %s\s*\{(.*?)\}\s*%s;" % (name, name), text, flags=re.S).group(1)
    nphi = c_defines("CAP_NPHI")["CAP_NPHI"]
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, rest = decl.split(None, 1)
        for item in rest.split(","):
            item = item.strip()
            m = re.match(r"(\w+)(?:\[(\w+)\])?$", item)
            n = 1
            if m.group(2):
                n = nphi if m.group(2) == "CAP_NPHI" else int(m.group(2))
            out.append((m.group(1).lower(), {"double": "c_double", "int": "c_int"}[ctype], n))
    return out


def shim():
    return fortran_statements(SHIM.read_text())


def module_part(stmts):
    end = stmts.index("end module cappgpu")
    return stmts[:end], stmts[end + 1:]


def fortran_parameters(stmts):
    vals = {}
    for s in stmts:
        if "parameter ::" in s:
            for name, v in re.findall(r"(\w+)\s*=\s*(-?\d+)", s.split("::", 1)[1]):
                vals[name.upper()] = int(v)
    return vals


def fortran_type_members(stmts, tname):
    i = stmts.index("type, bind(c) :: " + tname)
    out = []
    for s in stmts[i + 1:]:
        if s.startswith("end type"):
            break
        kind = re.match(r"(real|integer)\((c_\w+)\)\s*::", s).group(2)
        for item in s.split("::", 1)[1].split(","):
            m = re.match(r"\s*(\w+)(?:\((\d+)\))?\s*$", item)
            out.append((m.group(1), kind, int(m.group(2)) if m.group(2) else 1))
    return out


def fortran_interfaces(stmts):
    """bind name -> (fortran name, [(dummy, decl dict)])"""
    mod, _ = module_part(stmts)
    i0, i1 = mod.index("interface"), mod.index("end interface")
    res, cur = {}, None
    for s in mod[i0 + 1:i1]:
        m = re.match(r"integer\(c_int\) function (\w+)\s*\(([^)]*)\)\s*bind\(c, name=\"(\w+)\"\)", s)
        if m:
            dummies = [d.strip() for d in m.group(2).split(",") if d.strip()]
            cur = (m.group(1), m.group(3), {d: None for d in dummies}, dummies)
            continue
        if s.startswith("end function"):
            res[cur[1]] = (cur[0], [(d, cur[2][d]) for d in cur[3]])
            cur = None
            continue
        if s.startswith("import"):
            continue
        m = re.match(r"(integer|real|type|character)\(([^)]*)\)(.*?)::(.*)", s)
        assert m, s
        base, kind, attrs, names = m.groups()
        attrs = [a.strip() for a in attrs.split(",") if a.strip()]
        for item in re.findall(r"(\w+)(\([^)]*\))?", names):
            name, dim = item
            cur[2][name] = {"base": base, "kind": kind.replace("kind=", ""), "value": "value" in attrs,
                            "intent": next((a for a in attrs if a.startswith("intent")), None), "dim": dim}
    return res


C_SCALARS = {("integer", "c_int"): {"int"}, ("integer", "c_int64_t"): {"int64_t"},
             ("integer", "c_long_long"): {"long long", "unsigned long long"},
             ("real", "c_double"): {"double"}}


def compatible(f, ctype):
    """A Fortran dummy declaration and a C parameter type pass the same
    thing: a value of the same C type, or an address of it."""
    if f["value"]:
        if f["base"] == "type" and f["kind"] == "c_ptr":
            return ctype.endswith("*")
        return ctype in C_SCALARS.get((f["base"], f["kind"]), set())
    if not ctype.endswith("*"):
        return False
    pointee = ctype[:-1].strip()
    const = pointee.startswith("const ")
    pointee = pointee.replace("const ", "")
    if const and f["intent"] not in ("intent(in)",):
        return False        # the C side promises not to write what Fortran lets it write back
    if f["base"] == "character":
        return pointee == "char" and f["kind"] == "c_char"
    if f["base"] == "type":
        return pointee == f["kind"]
    return pointee in C_SCALARS.get((f["base"], f["kind"]), set())


def test_statement_reader_joins_continuations():
    st = fortran_statements("  call f(a, & ! note\n     & b)\n! only a comment\nx = 'a!b' ! c\n")
    assert st == ["call f(a, b)", "x = 'a!b'"]


def test_field_ids_and_codes_match_the_header():
    params = fortran_parameters(shim())
    fields = c_enum_values("cappgpu_field")
    cap = {k: v for k, v in params.items() if k.startswith("CAP_")}
    assert len(cap) >= 80
    for k, v in cap.items():
        assert fields[k] == v, k
    solvers = c_defines("CAPPGPU_SOLVER_")
    for k, v in solvers.items():
        assert params[k.replace("CAPPGPU_", "")] == v, k
    assert params["CAPPGPU_NOT_CONVERGED"] == c_defines("CAPPGPU_NOT_CONVERGED")["CAPPGPU_NOT_CONVERGED"]


@pytest.mark.parametrize("tname", ["cappgpu_params", "cappgpu_solve_report"])
def test_bind_c_types_match_the_header_structs(tname):
    assert fortran_type_members(shim(), tname) == c_struct_members(tname)


def test_every_interface_matches_its_c_prototype():
    protos = c_prototypes()
    ifaces = fortran_interfaces(shim())
    assert len(ifaces) >= 35
    for cname, (fname, dummies) in ifaces.items():
        assert fname == cname, (fname, cname)
        assert cname in protos, f"{cname} is not declared in the header"
        ctypes_ = protos[cname]
        assert len(dummies) == len(ctypes_), (cname, dummies, ctypes_)
        for (d, decl), ct in zip(dummies, ctypes_):
            assert decl is not None, (cname, d, "undeclared dummy")
            assert compatible(decl, ct), (cname, d, decl, ct)


def test_every_library_call_in_the_shim_is_bound():
    stmts = shim()
    ifaces = fortran_interfaces(stmts)
    mod, rest = module_part(stmts)
    i1 = mod.index("end interface")
    calls = set()
    for s in mod[i1:] + rest:
        calls |= set(re.findall(r"\b(cappgpu_\w+)\s*\(", s))
    procs = {m for s in stmts for m in re.findall(r"^subroutine (\w+)", s)}
    unbound = {c for c in calls if c not in ifaces and c not in procs}
    assert not unbound, unbound


def test_dropins_keep_the_reference_names_and_dummies():
    _, rest = module_part(shim())
    subs = {}
    for s in rest:
        m = re.match(r"subroutine (\w+)\s*(?:\(([^)]*)\))?\s*$", s)
        if m:
            subs[m.group(1)] = [d.strip() for d in (m.group(2) or "").split(",") if d.strip()]
    for ref_file, (name, dummies) in REFERENCE_DROPINS.items():
        assert name in subs, f"no drop-in for {ref_file}"
        assert subs[name] == dummies, (ref_file, subs[name], dummies)


def test_header_comment_lists_only_files_with_dropins():
    head = []
    for line in SHIM.read_text().splitlines():
        if line.startswith("module "):
            break
        head.append(line.lstrip("! "))
    claimed = set(re.findall(r"([\w\-*]+\.f90)", " ".join(head))) - {"cappgpu_iface.f90"}
    assert claimed == set(REFERENCE_DROPINS), claimed ^ set(REFERENCE_DROPINS)
