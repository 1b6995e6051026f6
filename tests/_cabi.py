"""Checks a ctypes binding against the prototypes of a C header.

Used by the CPU tests of libgsfft.so (include/gsfft.h) and of the oracle
library (oracle/sfft_oracle.h): for every function the binding declares, the
argument count and, per argument, the calling-convention class (pointer, or
an integer's width and signedness, or a floating type) must be the header's.
ctypes passes an argument by what argtypes says, so an int where the header
says long long, or a float where it says double, hands the callee undefined
bits without any error.
"""
import ctypes as C
import re


def header_prototypes(path):
    """{name: (return type, [argument types])} of the functions a C header
    declares (comments and preprocessor lines removed)."""
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//.*", "", txt)
    txt = re.sub(r"^\s*#.*$", "", txt, flags=re.M)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w \*]*?)\b(\w+)\s*\(([^;{}()]*)\)\s*;", txt, flags=re.S):
        ret, name, args = " ".join(m.group(1).split()), m.group(2), m.group(3)
        types = []
        for a in (" ".join(x.split()) for x in args.split(",")):
            if not a or a == "void":
                continue
            # drop the parameter name; keep pointer stars
            types.append(a if a.endswith("*") else re.sub(r"\s*\b\w+$", "", a))
        out[name] = (ret.strip(), types)
    return out


_SCALARS = {"int": ("int", 4, True), "unsigned": ("int", 4, False),
            "unsigned int": ("int", 4, False), "long": ("int", C.sizeof(C.c_long), True),
            "long long": ("int", 8, True), "size_t": ("int", C.sizeof(C.c_size_t), False),
            "double": "f64", "float": "f32", "void": "void"}


def c_kind(t, handles=()):
    """Calling-convention class of a C type (handles: pointer typedefs)."""
    t = t.replace("const ", "").strip()
    if "*" in t or t in handles:
        return "ptr"
    return _SCALARS[t]


def ctypes_kind(t):
    if t is None:
        return "void"
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return "ptr"
    if t is C.c_double:
        return "f64"
    if t is C.c_float:
        return "f32"
    return ("int", C.sizeof(t), t(-1).value < 0)


def check_binding(lib, header, handles=()):
    """Asserts that every bound function of `lib` (argtypes set) matches the
    header; returns (functions checked, header functions left unbound)."""
    protos = header_prototypes(header)
    checked, unbound = 0, []
    for name, (ret, args) in sorted(protos.items()):
        f = getattr(lib, name)
        if f.argtypes is None:
            unbound.append(name)
            continue
        assert len(f.argtypes) == len(args), (name, args)
        for i, (ct, pt) in enumerate(zip(args, f.argtypes)):
            assert c_kind(ct, handles) == ctypes_kind(pt), (name, i, ct, pt)
        assert c_kind(ret, handles) == ctypes_kind(f.restype), (name, ret, f.restype)
        checked += 1
    return checked, unbound
