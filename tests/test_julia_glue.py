"""The Julia glue package (julia/src/LatticeModelsGB300.jl) against the C header include/lmgpu.h
and against the reference API it plugs into.

Julia is not installed here, so the glue cannot be run; these tests read it as text and check
every `ccall` against the header declaration it binds: the function exists, the number of
arguments agrees, and each argument and the return value have a Julia type of the right
width and kind (pointer or scalar).  A wrong count or width in a ccall corrupts the stack on
the first call, so this is the check that matters most for the glue.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lmgpu.h")
JL = os.path.join(ROOT, "latticemodels.jl_gb300", "julia")
GLUE = os.path.join(JL, "src", "LatticeModelsGB300.jl")
EXT = os.path.join(JL, "ext", "LatticeModelsGB300ChainRulesCoreExt.jl")
PROJECT = os.path.join(JL, "Project.toml")

# C scalar type -> Julia types of the same width
SCALARS = {
    "int": {"Cint", "Int32"},
    "int64_t": {"Int64"},
    "double": {"Cdouble", "Float64"},
    "size_t": {"Csize_t", "UInt64"},
    "unsigned long long": {"Culonglong", "UInt64"},
}
TYPE_WORDS = {"int", "long", "unsigned", "double", "float", "char", "short", "int64_t", "size_t", "void"}
POINTER_JL = re.compile(r"^(Ptr|Ref)\{.*\}$|^Cstring$")


def _strip_comments(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def header_decls():
    text = _strip_comments(open(HEADER).read())
    decls = {}
    for m in re.finditer(r"\b((?:const\s+)?[A-Za-z_0-9]+\s*\**)\s*\b(lm_[a-z_0-9]+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        ret, name, args = m.group(1).strip(), m.group(2), " ".join(m.group(3).split())
        params = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        decls[name] = (ret, params)
    return decls


def _split_top(s):
    """Split a Julia tuple body at top-level commas."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def glue_ccalls():
    text = open(GLUE).read() + open(EXT).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(lm_[a-z_0-9]+), LIB\),\s*([A-Za-z0-9{}]+),\s*\(", text):
        # the argument-type tuple starts at m.end() - 1; find its matching parenthesis
        i, depth = m.end() - 1, 0
        for j in range(i, len(text)):
            if text[j] == "(":
                depth += 1
            elif text[j] == ")":
                depth -= 1
                if depth == 0:
                    break
        types = _split_top(text[i + 1:j])
        line = text.count("\n", 0, m.start()) + 1
        calls.append((m.group(1), m.group(2), types, line))
    return calls


def _c_kind(ctype):
    if "*" in ctype:
        return "ptr", None
    words = [w for w in ctype.replace("const", " ").split() if w]
    # a named parameter: "int ndof" -> "int", "unsigned long long seed" -> "unsigned long long"
    if len(words) > 1 and words[-1] not in TYPE_WORDS:
        words = words[:-1]
    return "scalar", " ".join(words)


def test_glue_present_and_has_ccalls():
    assert os.path.exists(GLUE)
    assert len(glue_ccalls()) >= 40


@pytest.mark.parametrize("name,ret,types,line", glue_ccalls(), ids=lambda v: str(v) if isinstance(v, (str, int)) else None)
def test_ccall_matches_header(name, ret, types, line):
    decls = header_decls()
    assert name in decls, f"line {line}: {name} is not declared in lmgpu.h"
    cret, params = decls[name]
    assert len(types) == len(params), \
        f"line {line}: {name} takes {len(params)} arguments in the header, the ccall passes {len(types)}"
    kind, base = _c_kind(cret)
    if kind == "ptr":
        assert POINTER_JL.match(ret), f"line {line}: {name} returns {cret}, ccall says {ret}"
    else:
        assert ret in SCALARS[base], f"line {line}: {name} returns {cret}, ccall says {ret}"
    for k, (jt, cp) in enumerate(zip(types, params)):
        kind, base = _c_kind(cp)
        if kind == "ptr":
            assert POINTER_JL.match(jt), f"line {line}: {name} argument {k + 1} is '{cp}', ccall passes {jt}"
        else:
            assert base in SCALARS, f"{name}: unknown C type {cp}"
            assert jt in SCALARS[base], f"line {line}: {name} argument {k + 1} is '{cp}', ccall passes {jt}"


def test_glue_binds_the_plugin_and_readout_entry_points():
    bound = {c[0] for c in glue_ccalls()}
    for fn in ("lm_solver_update", "lm_solver_step", "lm_localdensity", "lm_bond_currents",
               "lm_ring_push_localdensity", "lm_ring_push_currents", "lm_ring_push_op_currents",
               "lm_ell_op_currents", "lm_state_upload", "lm_state_download", "lm_kpm_moments",
               "lm_cheb_apply", "lm_ham_lanczos_bounds", "lm_state_set_weights", "lm_trace"):
        assert fn in bound, fn


# Base functions a module must qualify (Base.f) to add methods to; defining them bare shadows
# Base and fails once the module has used the Base binding.
BASE_FUNCS = {"take!", "put!", "push!", "pop!", "append!", "copy", "size", "length", "getindex", "setindex!",
              "show", "print", "close", "wait", "fill!", "resize!", "empty!", "isready", "reset"}
SPARSE_FUNCS = ("nnz", "nzrange", "rowvals", "nonzeros", "sparse", "spzeros", "findnz")


def test_glue_imports_and_definitions():
    text = open(GLUE).read()
    m = re.search(r"^using SparseArrays:(.*)$", text, re.M)
    imported = {w.strip() for w in m.group(1).split(",")} if m else set()
    for f in SPARSE_FUNCS:
        if re.search(r"(?<![\w.])" + f + r"\(", text):
            assert f in imported, f"{f} is used but not imported from SparseArrays"
    defined = set(re.findall(r"^function ([A-Za-z_][\w!]*)\(", text, re.M))
    defined |= set(re.findall(r"^([A-Za-z_][\w!]*)\([^)]*\)\s*=", text, re.M))
    assert not (defined & BASE_FUNCS), f"unqualified Base functions defined: {defined & BASE_FUNCS}"


# --- the drop-in surface: methods of the reference's own functions -------------------------
def _code(path=GLUE):
    """The file with comments and docstrings removed."""
    text = open(path).read()
    text = re.sub(r'"""(.*?)"""', " ", text, flags=re.S)
    return re.sub(r"#[^\n]*", " ", text)


def test_builder_hooks_into_construct_operator():
    """tightbinding_hamiltonian(GPUBuilder, l; t1, field) reaches the reference's builder hook
    construct_operator(BT::Type, sys::System, args...; field, auto_pbc_field)
    (src/operators/constructoperator.jl:136, :190-194) and returns an Operator whose data is the
    device Hamiltonian, which construct_hamiltonian wraps in the reference's Hamiltonian."""
    code = _code()
    assert re.search(r"struct GPUBuilder end", code)
    m = re.search(r"function LatticeModels\.construct_operator\(::Type\{GPUBuilder\}, sys::LatticeModels\.System, "
                  r"args\.\.\.;\s*field=LatticeModels\.NoField\(\), auto_pbc_field=true", code)
    assert m, "construct_operator(::Type{GPUBuilder}, sys, args...; field, auto_pbc_field) is missing"
    body = code[m.end():code.index("\nend\n", m.end())]
    assert "NearestNeighbor{1}" in body and "LatticeValue" in body
    assert "QuantumOpticsBase.Operator(LatticeModels.basis(sys), H)" in body
    assert "struct DeviceHamiltonian <: AbstractMatrix{ComplexF64}" in code


def test_readouts_are_methods_of_the_reference_functions():
    code = _code()
    imported = re.search(r"^import LatticeModels:(.*?)\n(?!\s)", code, re.M | re.S).group(1)
    for f in ("update_solver!", "step!", "evolution_cache", "localdensity", "densitymatrix", "Currents",
              "DensityCurrents"):
        assert re.search(r"(?<![\w!])" + re.escape(f) + r"(?![\w!])", imported), f"{f} is not imported from LatticeModels"
    # localdensity on device-backed Ket/Operator states returns the reference's LatticeValue
    m = re.search(r"function localdensity\(state::Union\{DeviceOperator,DeviceKet\}\)(.*?)\nend", code, re.S)
    assert m and "LatticeModels.LatticeValue(l," in m.group(1)
    assert re.search(r"const DeviceOperator = QuantumOpticsBase\.Operator\{<:Any,<:Any,<:DeviceState\}", code)
    assert re.search(r"const DeviceKet = QuantumOpticsBase\.Ket\{<:Any,<:DeviceVector\}", code)
    # DensityCurrents(H, P): the reference's lazy struct, specialised getindex and Currents
    assert re.search(r"const GPUDensityCurrents = DensityCurrents\{<:LatticeModels\.Hamiltonian\{<:Any,<:Any,"
                     r"<:DeviceHamiltonian\},", code)
    assert re.search(r"function Base\.getindex\(curr::GPUDensityCurrents, i::Int, j::Int\)", code)
    assert re.search(r"function Currents\(curr::GPUDensityCurrents\)", code)
    assert "LatticeModels.CURRENTS_EPS" in code
    # tr and copy of a device state (the reference's Evolution copies its states)
    assert re.search(r"LinearAlgebra\.tr\(st::DeviceState\) =", code)
    assert re.search(r"function Base\.copy\(s::DeviceState\)", code)
    assert re.search(r"Base\.copy\(v::DeviceVector\)", code)
    # densitymatrix on a GPUBuilder Hamiltonian: the device eigensystem at T = 0
    m = re.search(r"function densitymatrix\(ham::LatticeModels\.Hamiltonian\{<:Any,<:Any,<:DeviceHamiltonian\};(.*?)\nend",
                  code, re.S)
    assert m and "GPUEigensystem(H)" in m.group(1) and "gpu_densitymatrix" in m.group(1)
    assert "QuantumOpticsBase.Operator(QuantumOpticsBase.basis(ham), st)" in m.group(1)
    # the plugin methods for both state kinds
    assert re.search(r"step!\(s::ChebyshevGPU, st::DeviceState, _cache\)", code)
    assert re.search(r"step!\(s::ChebyshevGPU, v::DeviceVector, cache\)", code)
    assert re.search(r"function update_solver!\(s::ChebyshevGPU, H::DeviceHamiltonian, dt, force=false\)", code)


def test_rrule_is_a_package_extension():
    """ChainRulesCore is a weak dependency: the rrule lives in ext/ and the module never
    imports ChainRulesCore itself."""
    assert "ChainRulesCore" not in _code()
    ext = _code(EXT)
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(density_loss\), V, B, p::DensityLossProblem\)", ext)
    proj = open(PROJECT).read()
    assert re.search(r"\[weakdeps\]\s*\nChainRulesCore = ", proj)
    assert re.search(r"\[extensions\]\s*\nLatticeModelsGB300ChainRulesCoreExt = \"ChainRulesCore\"", proj)
    # the reference package's own uuid (its Project.toml) is the dependency
    assert 'LatticeModels = "3c3db7f8-440c-4375-905c-1a18b5307bed"' in proj
