"""The Fortran drop-in layer (fortran/*.f90), checked without a Fortran
compiler (there is none on either machine).

* fortran/fair_gpu.f90 binds every entry point of include/*.h: the same
  names (bind(C) label = interface name), each exported by
  libfair_gb300.so, the same number of arguments, and per argument the same
  passing (VALUE for C scalars, by reference or TYPE(C_PTR), VALUE for C
  pointers) and interoperable kind (c_int32_t <-> int32_t, ...);
* the forwarding modules (sparse_matrices.f90, system_generation.f90,
  airms.f90) call only bound entry points, each with its number of
  arguments, and keep the reference's public procedures with their dummy
  argument names (sparse_matrices.f90:50-176 and :180-831,
  system_generation.f90:17-745, AIRMs.f90:6-1212).
"""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FDIR = os.path.join(ROOT, "fortran")

C_SCALAR = {"int32_t": "c_int32_t", "int64_t": "c_int64_t", "uint64_t": "c_int64_t",
            "int": "c_int", "double": "c_double", "float": "c_float", "char": "c_char",
            "fair_opts": "fair_opts", "fair_data": "fair_data"}
HANDLES = {"fair_csr", "fair_batch", "fair_mf"}


# ------------------------------------------------------------------ C side ----
def c_prototypes():
    out = {}
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"((?:const\s+)?[A-Za-z_0-9]+\s*\**)\s*(fair_[a-z0-9_]+)\s*\(([^)]*)\)\s*;",
                             text):
            ret, name, params = m.group(1), m.group(2), " ".join(m.group(3).split())
            args = [] if params in ("", "void") else [c_arg(p) for p in params.split(",")]
            out[name] = ("c_ptr" if "*" in ret else "c_int", args)
    return out


def c_arg(p):
    p = p.replace("const", " ").strip()
    stars = p.count("*")
    base = p.replace("*", " ").split()[0]
    if base in HANDLES:
        return ("ptr", None) if stars == 0 else ("ref", "c_ptr")
    if stars == 0:
        return ("val", C_SCALAR[base])
    if base == "void":
        return ("ptr", None)
    return ("ref", C_SCALAR[base])


# ------------------------------------------------------------ Fortran side ----
def logical_lines(path):
    """Source lines with comments removed and continuations joined."""
    lines, buf = [], ""
    for raw in open(path):
        line = raw.rstrip("\n")
        q = None
        for i, ch in enumerate(line):
            if ch in "'\"":
                q = None if q == ch else (ch if q is None else q)
            elif ch == "!" and q is None:
                line = line[:i]
                break
        line = line.strip()
        if buf:
            line = line[1:].strip() if line.startswith("&") else line
        if line.endswith("&"):
            buf += line[:-1] + " "
            continue
        lines.append(buf + line)
        buf = ""
    return [ln for ln in lines if ln]


def f_bindings():
    out = {}
    lines = logical_lines(os.path.join(FDIR, "fair_gpu.f90"))
    i = 0
    while i < len(lines):
        m = re.match(r"(integer\(c_int\)|type\(c_ptr\)|integer\(c_size_t\))\s+function\s+(\w+)\s*"
                     r"\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", lines[i], re.I)
        if not m:
            i += 1
            continue
        ret, name, dummies, label = m.groups()
        assert name == label or not name.startswith("fair_"), \
            f"{name} is bound to the C name {label}"
        dummies = [d.strip() for d in dummies.split(",") if d.strip()]
        decl = {}
        i += 1
        while not lines[i].lower().startswith("end function"):
            d = re.match(r"([a-z]+\([^)]*\))\s*((?:,\s*[a-z]+(?:\([^)]*\))?\s*)*)::\s*(.+)$",
                         lines[i], re.I)
            if d:
                tspec, attrs, names = d.groups()
                kind = re.search(r"\((?:kind=)?(\w+)\)", tspec).group(1).lower()
                value = "value" in attrs.lower()
                for nm in re.findall(r"(\w+)\s*(\(\*\))?", names):
                    decl[nm[0]] = (kind, value, bool(nm[1]))
            i += 1
        args = []
        for dname in dummies:
            assert dname in decl, f"{name}: dummy {dname} has no declaration"
            kind, value, _ = decl[dname]
            if value:
                args.append(("ptr", None) if kind == "c_ptr" else ("val", kind))
            else:
                args.append(("ref", kind))
        out[name] = ("c_ptr" if ret.lower().startswith("type") else ret.lower()[8:-1], args, dummies)
        i += 1
    return out


def compatible(f, c):
    if f == ("ptr", None):  # TYPE(C_PTR), VALUE carries any C pointer
        return c[0] in ("ptr", "ref")
    return f == c


def test_every_header_entry_is_bound_with_matching_arguments():
    C = c_prototypes()
    F = {k: v for k, v in f_bindings().items() if k.startswith("fair_")}
    assert len(C) >= 80
    assert sorted(C) == sorted(F), (set(C) ^ set(F))
    bad = []
    for name, (cret, cargs) in C.items():
        fret, fargs, dummies = F[name]
        if cret != fret or len(cargs) != len(fargs):
            bad.append((name, "return or argument count", cret, fret, len(cargs), len(fargs)))
            continue
        for k, (ca, fa) in enumerate(zip(cargs, fargs)):
            if not compatible(fa, ca):
                bad.append((name, dummies[k], ca, fa))
    assert not bad, bad


def test_bound_names_are_exported(fair):
    L = fair.lib()
    missing = [n for n in f_bindings() if n.startswith("fair_") and not hasattr(L, n)]
    assert not missing, missing


def call_args(text, start):
    """Top-level comma-separated arguments of the call whose '(' is at start."""
    depth, args, cur, q = 0, [], "", None
    for ch in text[start:]:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
            cur += ch
            continue
        if ch == "(":
            depth += 1
            if depth == 1:
                continue
        elif ch == ")":
            depth -= 1
            if depth == 0:
                if cur.strip():
                    args.append(cur.strip())
                return args
        elif ch == "," and depth == 1:
            args.append(cur.strip())
            cur = ""
            continue
        cur += ch
    raise AssertionError("unbalanced call")


@pytest.mark.parametrize("module", ["sparse_matrices.f90", "system_generation.f90", "airms.f90"])
def test_forwarding_calls_match_bindings(module):
    F = f_bindings()
    text = "\n".join(logical_lines(os.path.join(FDIR, module)))
    calls = 0
    for m in re.finditer(r"\b(fair_[a-z0-9_]+)\s*\(", text):
        name = m.group(1)
        if name in ("fair_check", "fair_cstr", "fair_status_text"):
            continue
        assert name in F, f"{module} calls unbound {name}"
        n = len(call_args(text, m.end() - 1))
        assert n == len(F[name][1]), f"{module}: {name} called with {n} arguments"
        calls += 1
    assert calls >= 5


# the reference's public procedures and their dummy arguments
REFERENCE_PROCS = {
    "sparse_matrices.f90": {
        "construct_csr_matrix": "m,n,vA,IA,JA,A", "construct_csc_matrix": "m,n,vA,IA,JA,A",
        "print_line": "A,k", "csr_matrowvec": "A,k,v", "sparsematmul": "A,v",
        "sparsetransmul": "A,v", "transposition": "A", "conv_to_CSC": "A", "conv_to_CSR": "A",
        "SM_set_element": "A,i,j,aij", "SM_delete_element": "A,i,j", "SM_get_element": "A,i,j",
        "compute_row_norms": "A,p", "compute_column_norms": "A,p",
        "add_mult_row": "A,k,c,w,lwrb,upb", "scalar_mult": "A,c"},
    "system_generation.f90": {
        "linspace": "a,b,n", "fanlineartomo": "dat,geometry_fix", "paralleltomo": "dat",
        "read_data": "dat,inputfile,verbose", "read_ref": "xref,inputfile,n,verbose",
        "read_ordering": "ordering,inputfile,verbose", "store_matrix": "A,inputfile,verbose",
        "read_csr_matrix": "A,inputfile,verbose", "read_csc_matrix": "A,inputfile,verbose",
        "add_white_noise": "bt,e,b,eta"},
    "airms.f90": {
        "initialise_options": "options", "set_upperbound": "options,ubound",
        "set_lowerbound": "options,lbound", "art": "Xout,art_method,A,b,Kin,x0,xref,order,options",
        "twin_art": "xout,final_it,Xstore,Ystore,EG,art_method,stoprule,A,b,Kin,x0,y0,order,"
                    "slack,options",
        "gradient_descent": "xout,A,b,max_iter,x0,rho_in,tolerance,options",
        "sirt": "xout,sirt_method,A,b,Kin,x0,options", "normest": "A,tolerance,max_its",
        "scramble": "number_of_values"},
}
TYPE_BOUND = {"matvecmul", "transvecmul", "rowvecmult", "print_part", "transpose",
              "convert_to_CSR", "convert_to_CSC", "set_element", "get_element",
              "delete_element", "row_norms", "column_norms", "multiply_by_scalar",
              "add_scalar_mult_row"}


@pytest.mark.parametrize("module", sorted(REFERENCE_PROCS))
def test_reference_procedures_kept(module):
    text = "\n".join(logical_lines(os.path.join(FDIR, module)))
    for proc, dummies in REFERENCE_PROCS[module].items():
        m = re.search(rf"(?:subroutine|function)\s+{proc}\s*\(([^)]*)\)", text, re.I)
        assert m, f"{module}: {proc} missing"
        got = ",".join(d.strip() for d in m.group(1).split(","))
        assert got == dummies, f"{module}: {proc}({got}) differs from the reference's ({dummies})"
    if module == "sparse_matrices.f90":
        bound = set(re.findall(r"procedure\s*::\s*(\w+)\s*=>", text, re.I))
        assert TYPE_BOUND <= bound, TYPE_BOUND - bound
        for t in ("sparse_matrix", "CSR_matrix", "CSC_matrix"):
            assert re.search(rf"type(?:,\s*extends\(\w+\))?\s*::\s*{t}\b|type\s+{t}\b", text, re.I)
    if module == "airms.f90":
        assert re.search(r"type\s+opts\b", text, re.I)
