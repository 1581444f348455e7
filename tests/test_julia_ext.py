"""CPU checks of the Julia package extension (mpskit.jl_gb300/ext/MPSKitGB300Ext.jl), which
cannot run here (no Julia): every method it adds to a function of the reference must be
strictly more specific, in its positional arguments, than the reference method it takes
over -- never an identical signature (a method overwrite, refused when an extension
precompiles) and never selected by a keyword (Julia does not dispatch on keywords).

The reference's positional signatures are listed below with their file:line (MPSKit.jl
v0.13.13); the subtype relations used are those of the reference's type definitions."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXT = os.path.join(ROOT, "mpskit.jl_gb300", "ext", "MPSKitGB300Ext.jl")

# reference methods (positional argument types; "Any" = untyped)
REFERENCE = {
    "AC_hamiltonian": [
        # src/algorithms/derivatives/hamiltonian_derivatives.jl:44-55
        ("Int", "_HAM_MPS_TYPES", "MPOHamiltonian", "_HAM_MPS_TYPES", "Any"),
        # src/algorithms/derivatives/mpo_derivatives.jl:46-55
        ("Int", "Any", "Any", "Any", "Any"),
        # hamiltonian_derivatives.jl:219-226 (WindowMPS forwarding)
        ("Int", "WindowMPS", "WindowMPOHamiltonian", "WindowMPS", "Any"),
    ],
    "AC2_hamiltonian": [
        ("Int", "_HAM_MPS_TYPES", "MPOHamiltonian", "_HAM_MPS_TYPES", "Any"),  # :206-217
        ("Int", "Any", "Any", "Any", "Any"),                                 # mpo_derivatives.jl:56-66
        ("Int", "WindowMPS", "WindowMPOHamiltonian", "WindowMPS", "Any"),
    ],
    "C_hamiltonian": [
        ("Int", "Any", "Any", "Any", "Any"),  # mpo_derivatives.jl:37-45
    ],
    "find_groundstate!": [
        # src/algorithms/groundstate/dmrg.jl:279-285 (envs has a default: 3- and 4-arg methods)
        ("AbstractFiniteMPS", "Any", "Union{DMRG, DMRG2}", "Any"),
        ("AbstractFiniteMPS", "Any", "Union{DMRG, DMRG2}"),
    ],
    "fixedpoint": [
        ("Any", "Any", "Symbol", "Lanczos"),  # src/algorithms/fixedpoint.jl:15-18
        ("Any", "Any", "Symbol", "Arnoldi"),  # :19-23
    ],
}

# direct supertypes (the reference's definitions); everything is below "Any"
SUPER = {
    "FiniteMPS{<:MPSTensor}": ["_HAM_MPS_TYPES", "AbstractFiniteMPS"],
    "InfiniteMPS{<:MPSTensor}": ["_HAM_MPS_TYPES"],
    "WindowMPS": ["AbstractFiniteMPS"],
    "FiniteMPOHamiltonian": ["MPOHamiltonian"],
    "InfiniteMPOHamiltonian": ["MPOHamiltonian"],
    "DMRG2{<:Any, <:Any, <:Any, <:GB300Backend}": ["Union{DMRG, DMRG2}"],
    "GB300Derivative": ["DerivativeOperator"],
}


def subtype(a, b):
    if a == b or b == "Any":
        return True
    return any(subtype(s, b) for s in SUPER.get(a, []))


def split_top(s, sep=","):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == sep and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return out


def ext_methods():
    """(name, positional types, keyword text) of every method the extension defines,
    with the @eval loop over (MPS, HAM, ENV) expanded."""
    src = open(EXT).read()
    aliases = dict(re.findall(r"^const (_\w+) = (\S+)$", src, flags=re.M))
    loops = re.findall(r"for \(MPS, HAM, ENV\) in \((.*?)\)\n\s+@eval", src, flags=re.S)
    combos = []
    for body in loops:
        for tup in re.findall(r"\(([^()]*)\)", body):
            combos.append([t.strip() for t in tup.split(",")])
    out = []
    for m in re.finditer(r"function (\w+!?)\(", src):
        name = m.group(1)
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        sig = src[m.end():i - 1]
        pos, _, kw = sig.partition(";")
        args, ndefault = [], 0
        for a in split_top(pos):
            ndefault += "=" in a
            a = a.split("=")[0].strip()
            t = a.split("::", 1)[1].strip() if "::" in a else "Any"
            args.append(t)
        # trailing positional defaults define the shorter methods too
        variants = [args[:len(args) - k] for k in range(ndefault + 1)]
        for args in variants:
            out.extend(_instances(name, args, combos, aliases, kw))
    return out


def _instances(name, args, combos, aliases, kw):
    insts = [args]
    if any(t.startswith("$") for t in args):
        insts = [[{"$MPS": mps, "$HAM": ham, "$ENV": env}.get(t, t) for t in args]
                 for mps, ham, env in combos]
    return [(name, tuple(aliases.get(t, t) for t in a), kw) for a in insts]


@pytest.mark.parametrize("name", sorted(REFERENCE))
def test_every_overload_out_specialises_the_reference(name):
    mine = [(a, kw) for n, a, kw in ext_methods() if n == name]
    assert mine, f"the extension defines no {name}"
    for args, kw in mine:
        beaten = False
        for ref in REFERENCE[name]:
            assert args != ref, f"{name}{args} overwrites a reference method"
            if len(ref) != len(args):
                continue
            le = all(subtype(a, r) for a, r in zip(args, ref))
            strict = le and any(a != r for a, r in zip(args, ref))
            if le:
                assert strict, f"{name}{args} is not strictly more specific than {ref}"
                beaten = True
        assert beaten, f"{name}{args} does not narrow any reference method of its arity"
        # a required GB300Backend keyword would make every default call throw
        assert not re.search(r"backend::GB300Backend\s*(,|$)", kw.strip()), kw


def test_non_gb300_backends_fall_back_to_the_reference():
    src = open(EXT).read()
    for name in ("AC_hamiltonian", "AC2_hamiltonian", "C_hamiltonian"):
        assert re.search(rf"return invoke\({name},", src), name
    assert "const CTX_LOCK = ReentrantLock()" in src and "lock(CTX_LOCK)" in src
