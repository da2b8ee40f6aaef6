#!/usr/bin/env python3
"""Generate tests/golden/reference_outputs.json by running the reference's
own Fortran routines (TEST INFRASTRUCTURE ONLY).

Usage (in the build container, where the reference sources are):
    python tests/golden/make_golden.py [--reference DIR] [--only REGEX]

For every case of golden_cases.py: build the seeded state, load it into the
reference's module arrays, run setind.f90 and then the case's reference
subroutine through f90exec (the reference's source, translated statement
by statement), and record a digest of every module array, the module
scalars and the unit-66 lines afterwards.  The reference directory is read
here only; the fixture it writes is all the tests need.
"""
import argparse
import hashlib
import json
import pathlib
import re
import sys
import time

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (HERE, HERE.parent, ROOT / "oracle", ROOT):
    sys.path.insert(0, str(p))

import numpy as np  # noqa: E402

import cappgpu  # noqa: E402
from cappgpu import FIELD_NAMES  # noqa: E402
import f90exec as F  # noqa: E402
import golden_cases as G  # noqa: E402
import oracle as O  # noqa: E402

OUT = HERE / "reference_outputs.json"


def module_array(ns, name):
    """The module array (or its component row) behind a field name."""
    if name in ("gradu", "gradv", "gradw", "gradp", "gradte", "graded"):
        return ns.get(name)
    if name.startswith("grad") and name[-2:] in ("_x", "_y", "_z"):
        return ns.get(name[:-2])[" xyz".index(name[-1])]
    return ns.get(G.FIELD_ALIASES.get(name, name))


def load_state(prog, ns, st):
    for name in FIELD_NAMES:
        module_array(ns, name)[1:] = st.field(name)
    for face in G.BC_FACES:
        b = st.bc(face)
        ns.get(face)[1:1 + b.size] = b
    for name, _ in type(st.params)._fields_:
        if name in G.BUILD_ONLY_PARAMS:
            continue
        v = getattr(st.params, name)
        mname = G.PARAM_ALIASES.get(name, name)
        sym = prog.mod[mname]
        if sym.rank:
            ns.get(mname)[1:1 + len(v)] = list(v)
        elif sym.typ == "l":
            ns.set(mname, bool(v))
        elif sym.typ == "i":
            ns.set(mname, int(v))
        else:
            ns.set(mname, F.F8(v))
    ns.set("imon", 3)
    ns.set("jmon", 3)
    ns.set("kmon", 3)
    # the build's configuration of the gradient switch (input file): Gauss
    ns.set("gauss", True)
    ns.set("lstsq", False)
    # module values init.f90 derives from the ones read (:273-274, 332-333)
    urf = ns.get("urf")
    with np.errstate(divide="ignore"):     # the unused slots (urf = 0) give Inf there too
        ns.get("urfr")[1:11] = [F.F4(1.0) / F.F8(x) for x in urf[1:11]]
    ns.get("urfm")[1:11] = [F.F4(1.0) - F.F8(x) for x in urf[1:11]]
    cmu25 = np.sqrt(np.sqrt(F.F8(ns.get("cmu"))))
    ns.set("cmu25", cmu25)
    ns.set("cmu75", cmu25 * cmu25 * cmu25)


def read_params(prog, ns, st):
    vals = {}
    for name, _ in type(st.params)._fields_:
        if name in G.BUILD_ONLY_PARAMS:
            continue
        mname = G.PARAM_ALIASES.get(name, name)
        sym = prog.mod[mname]
        v = ns.get(mname)
        if sym.rank:
            vals[name] = [float(x) if sym.typ in ("r4", "r8") else int(x) for x in v[1:11]]
        elif sym.typ == "l":
            vals[name] = int(bool(v))
        elif sym.typ == "i":
            vals[name] = int(v)
        else:
            vals[name] = float(v)
    return G.params_record(vals)


def run_case(ref, c):
    grid_case, st = c.build(O)
    inputs = G.state_digest(st)
    before = {n: G.field_digest(st.field(n)) for n in FIELD_NAMES}
    params_before = G.oracle_params(st)
    prog = F.Program((ref / "modules_allocatable.f90").read_text())
    for f in ["setind.f90"] + list(c.files):
        f, only = (f, None) if isinstance(f, str) else (f[0], set(f[1]))
        prog.add_source((ref / f).read_text(), only=only, include_dir=ref)
    for name, parts in c.snippets:
        if isinstance(parts, str):
            parts = [parts]
        text = "\n".join(x if isinstance(x, str) else
                         "\n".join((ref / x[0]).read_text().splitlines()[x[1] - 1:x[2]]) for x in parts)
        prog.add_snippet(name, text, include_dir=ref)
    for q, (f, a, b) in enumerate(c.setup):
        prog.add_snippet(f"setup{q}", "\n".join((ref / f).read_text().splitlines()[a - 1:b]), include_dir=ref)
    prog.compile(stubs=c.stubs)
    ns = prog.namespace(st.dims)
    load_state(prog, ns, st)
    for k, v in c.switches.items():
        ns.set(k, v)
    ns.call("setind")
    for q in range(len(c.setup)):
        ns.call(f"setup{q}")
    li, lk = ns.get("li")[1:st.dims[0] + 1], ns.get("lk")[1:st.dims[2] + 1]
    if not (np.array_equal(li, st.li()) and np.array_equal(lk, st.lk())):
        raise AssertionError(f"{c.name}: setind index maps differ from the oracle's")
    calls = G.reference_calls(c, grid_case)
    t = time.time()
    for sub, args in calls:
        ns.call(sub, *[module_array(ns, a) if isinstance(a, str) else a for a in args])
    dt = time.time() - t
    after = {n: G.field_digest(module_array(ns, n)[1:]) for n in FIELD_NAMES}
    used = ["modules_allocatable.f90", "setind.f90"] + [f if isinstance(f, str) else f[0] for f in c.files]
    used += [f for f, _, _ in c.setup]
    for _, parts in c.snippets:
        for x in ([parts] if isinstance(parts, str) else parts):
            if isinstance(x, tuple):
                used.append(x[0])
            else:
                used += re.findall(r"include '([^']+)'", x)
    for f in list(used):                  # files that INCLUDE lines of those bring in
        for line in (ref / f).read_text().splitlines():
            m = re.match(r"\s*include\s+'([^']+)'", line, re.I)
            if m and (ref / m.group(1)).exists():
                used.append(m.group(1))
    sources = {f: hashlib.sha256((ref / f).read_bytes()).hexdigest()[:16] for f in sorted(set(used))}
    params = read_params(prog, ns, st)
    return {
        "routine": [sub for sub, _ in calls], "inputs": inputs,
        # the reference source files this record was computed from (sha256)
        "sources": sources,
        # digests of the arrays the routine changed, and one over all arrays
        "fields": {n: d for n, d in after.items() if d != before[n]},
        "all_fields": G.all_fields_digest(after),
        # the module scalars it changed, and a digest over all of them
        "params": {k: v for k, v in params.items() if v != params_before[k]},
        "all_params": G.params_digest(params),
        "unit66": ns.units.get(66, []),
        "li": [int(x) for x in li], "lk": [int(x) for x in lk],
        "ijkpr": int(ns.get("ijkpr")),
    }, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    ref = pathlib.Path(a.reference)
    O.build()
    out = json.loads(OUT.read_text()) if OUT.exists() and a.only else {}
    for c in G.all_cases():
        if a.only and not re.search(a.only, c.name):
            continue
        rec, dt = run_case(ref, c)
        out[c.name] = rec
        # immediate comparison with the oracle, for the generator's log
        grid_case, st = c.build(O)
        G.run_oracle(c, grid_case, st)
        got = {n: G.field_digest(st.field(n)) for n in FIELD_NAMES}
        diff = [n for n, d in rec["fields"].items() if got[n] != d]
        if G.all_fields_digest(got) != rec["all_fields"]:
            diff.append("(all arrays)")
        op = G.oracle_params(st)
        pdiff = [k for k, v in rec["params"].items() if op[k] != v]
        if G.params_digest(op) != rec["all_params"]:
            pdiff.append("(all scalars)")
        print(f"{c.name:48s} {dt:7.2f}s  fields differing: {diff or 'none'}  params differing: {pdiff or 'none'}",
              flush=True)
    lines = [f"{json.dumps(k)}: {json.dumps(out[k], sort_keys=True, separators=(',', ':'))}" for k in sorted(out)]
    OUT.write_text("{\n" + ",\n".join(lines) + "\n}\n")      # one case per line
    print("wrote", OUT, len(out), "cases")


if __name__ == "__main__":
    main()
