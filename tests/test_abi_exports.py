"""The C-ABI library builds for sm_103a, loads without a GPU, and exports
every entry point that include/swap_gpu.h declares (no compute calls)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def header_symbols():
    text = (ROOT / "include" / "swap_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(swap_[a-zA-Z0-9_]+)\s*\(", text)))


def test_header_declares_entries():
    syms = header_symbols()
    for s in ("swap_init", "swap_get_interp_weights", "swap_update_np", "swap_update_up", "swap_get_Ep",
              "swap_predict_B", "swap_correct_B", "swap_check_time_step", "swap_ion_step"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from swap_gb300 import build

    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert lib.swap_abi_version() == 1


def test_python_binding_covers_header():
    from swap_gb300 import abi

    assert set(header_symbols()) <= set(abi.SIGNATURES), set(header_symbols()) - set(abi.SIGNATURES)


def test_kernels_compiled_for_sm103a_only():
    from swap_gb300 import build

    flags = " ".join(build.ARCH)
    assert "compute_103a" in flags and "sm_103a" in flags
    assert "sm_100" not in flags and "sm_90" not in flags


def test_fortran_module_binds_declared_symbols():
    """Every bind(C) name of the Fortran interface module is an entry the
    header declares (so a SWAP build that uses the module links)."""
    text = (ROOT / "swap_gb300" / "fortran" / "swap_gpu_iface.f90").read_text()
    names = set(re.findall(r'bind\(C,\s*name="(swap_[A-Za-z0-9_]+)"\)', text))
    assert len(names) > 30
    missing = names - set(header_symbols())
    assert not missing, missing


def test_header_compiles_as_c_and_links(tmp_path):
    """A C caller (what a Fortran ISO_C_BINDING build links like) compiles
    against the header with every warning an error, links every declared
    entry from the library, and runs without a GPU."""
    import shutil
    import subprocess

    from swap_gb300 import build

    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest

        pytest.skip("no C compiler")
    lib_path = build.build()
    syms = header_symbols()
    src = tmp_path / "caller.c"
    src.write_text(
        '#include <stdio.h>\n#include "swap_gpu.h"\n'
        "typedef void (*entry)(void);\n"
        "static const entry entries[] = {\n" + "".join(f"  (entry){s},\n" for s in syms) + "};\n"
        "int main(void) {\n"
        '  printf("%d %d\\n", (int)(sizeof entries / sizeof entries[0]), swap_abi_version());\n'
        "  return 0;\n}\n")
    exe = tmp_path / "caller"
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Wpedantic", "-Werror", f"-I{ROOT / 'include'}",
                        str(src), f"-L{lib_path.parent}", f"-l:{lib_path.name}", f"-Wl,-rpath,{lib_path.parent}",
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == [str(len(syms)), "1"]


# ---- the Fortran interfaces against the header's prototypes ----

def _header_prototypes():
    """{name: (return type, [parameter types])} with pointer and array
    parameters written as 'T*'."""
    text = (ROOT / "include" / "swap_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"^([A-Za-z_][A-Za-z0-9_ *]*?)\b(swap_\w+)\s*\(([^;]*?)\)\s*;", text,
                                      flags=re.M | re.S):
        types = []
        for a in (x.strip() for x in args.replace("\n", " ").split(",")):
            if not a or a == "void":
                continue
            arr = a.endswith("]")
            a = re.sub(r"\[[^\]]*\]$", "", a).strip()
            t = re.match(r"^(.*?)\w+$", a).group(1)
            types.append(re.sub(r"\s+", " ", t).strip().replace(" *", "*").replace("const ", "") + ("*" if arr else ""))
        out[name] = (re.sub(r"\s+", " ", ret).strip().replace(" *", "*"), types)
    return out


def _fortran_interfaces():
    """{bind name: (result type, [(dummy, type spec with attributes)])} of the
    interface blocks, continuation lines joined and comments dropped."""
    lines, buf = [], ""
    for raw in (ROOT / "swap_gb300" / "fortran" / "swap_gpu_iface.f90").read_text().splitlines():
        s = raw.split("!")[0].rstrip()
        if not s.strip():
            continue
        s = (buf + " " + s.strip().lstrip("&").strip()) if buf else s.strip()
        if s.endswith("&"):
            buf = s[:-1].rstrip()
            continue
        buf = ""
        lines.append(s)
    out, i = {}, 0
    while i < len(lines):
        m = re.match(r'^(.*?)\bfunction\s+\w+\s*\(([^)]*)\)\s*bind\(C,\s*name="(\w+)"\)', lines[i], re.I)
        if m:
            decl, i = {}, i + 1
            while not re.match(r"^end\s+function", lines[i], re.I):
                d = re.match(r"^(?!import)(.*?)::(.*)$", lines[i], re.I)
                if d:
                    for nm in re.findall(r"(\w+)\s*(?:\([^)]*\))?", d.group(2)):
                        decl[nm.lower()] = d.group(1).strip().lower()
                i += 1
            dummies = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
            out[m.group(3)] = (m.group(1).strip().lower(), [(a, decl.get(a, "")) for a in dummies])
        i += 1
    return out


_BY_VALUE = {"int32_t": {"integer(c_int32_t)", "integer(c_int)"}, "int": {"integer(c_int)", "integer(c_int32_t)"},
             "uint32_t": {"integer(c_int32_t)"}, "int64_t": {"integer(c_int64_t)"},
             "uint64_t": {"integer(c_int64_t)"}, "double": {"real(c_double)"}, "float": {"real(c_float)"},
             "swap_exchange_fn": {"type(c_funptr)"}}
_BY_REFERENCE = {"double": {"real(c_double)", "real(wp)"}, "float": {"real(c_float)", "real(wp)"},
                 "int32_t": {"integer(c_int32_t)", "integer(c_int)"}, "int64_t": {"integer(c_int64_t)"},
                 "char": {"character(kind=c_char)"}, "swap_ctx*": {"type(c_ptr)"},
                 "swap_surrogate*": {"type(c_ptr)"}}


def test_fortran_interfaces_match_the_header_prototypes():
    """Every bind(C) interface passes each argument as the C prototype takes
    it: scalars by value with the same kind, pointers as `type(c_ptr),
    value` or by reference to an object of the pointed-to type (real(wp)
    arrays for the real arrays, whose width swap_dims.real_bytes gives)."""
    protos, ifaces = _header_prototypes(), _fortran_interfaces()
    assert len(ifaces) > 30
    bad = []
    for name, (result, dummies) in ifaces.items():
        ret, types = protos[name]
        if len(types) != len(dummies):
            bad.append((name, "takes", len(types), "arguments, the interface", len(dummies)))
            continue
        if not result.startswith({"int": "integer(c_int)", "const char*": "type(c_ptr)"}[ret]):
            bad.append((name, "returns", ret, result))
        for ctype, (dummy, spec) in zip(types, dummies):
            by_value = "value" in spec
            base = spec.split(",")[0].replace(" ", "")
            if ctype.endswith("*"):
                pointee = ctype[:-1]
                ok = base == "type(c_ptr)" if by_value else (
                    pointee == "void" or base in _BY_REFERENCE.get(pointee, {f"type({pointee}_t)"}))
            else:
                ok = by_value and base in _BY_VALUE.get(ctype, ())
            if not ok:
                bad.append((name, dummy, ctype, spec))
    assert not bad, bad


# ---- the argument structs: C, ctypes and Fortran layouts ----

_STRUCTS = {"swap_dims": ("Dims", "swap_dims_t"), "swap_params": ("Params", "swap_params_t"),
            "swap_coords": ("Coords", "swap_coords_t"), "swap_sources": ("Sources", "swap_sources_t"),
            "swap_diag_spec": ("DiagSpec", "swap_diag_spec_t"), "swap_load_spec": ("LoadSpec", None)}


def _c_struct_fields():
    """{struct: [(field, C type)]} from the header's typedefs."""
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "swap_gpu.h").read_text(), flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (swap_\w+) \{(.*?)\}", text, flags=re.S):
        fields = []
        for decl in (d.strip() for d in body.split(";") if d.strip()):
            m = re.match(r"^((?:const )?\w+)\s*(.*)$", " ".join(decl.split()))
            for f in m.group(2).split(","):
                f = f.strip()
                fields.append((f.lstrip("*"), m.group(1) + "*" * f.count("*")))
        out[name] = fields
    return out


def test_struct_layouts_agree_in_c_ctypes_and_fortran(tmp_path):
    """The C compiler's offsets and sizes of every argument struct equal the
    ctypes mirrors', and each Fortran bind(C) type lists the same fields in
    the same order with interoperable kinds."""
    import shutil
    import subprocess

    from swap_gb300 import abi

    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest

        pytest.skip("no C compiler")
    cfields = _c_struct_fields()
    assert set(_STRUCTS) <= set(cfields)
    prog = ['#include <stddef.h>', '#include <stdio.h>', '#include "swap_gpu.h"', "int main(void) {"]
    for s in _STRUCTS:
        prog.append(f'  printf("{s} %zu\\n", sizeof({s}));')
        prog += [f'  printf("{s}.{f} %zu\\n", offsetof({s}, {f}));' for f, _ in cfields[s]]
    prog += ["  return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(prog) + "\n")
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    c_layout = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                             check=True).stdout.splitlines())
    ftext = (ROOT / "swap_gb300" / "fortran" / "swap_gpu_iface.f90").read_text()
    fkind = {"int32_t": "integer(c_int32_t)", "uint32_t": "integer(c_int32_t)", "int64_t": "integer(c_int64_t)",
             "uint64_t": "integer(c_int64_t)", "double": "real(c_double)", "const double*": "type(c_ptr)"}
    for s, (py, ftype) in _STRUCTS.items():
        cls = getattr(abi, py)
        assert [f for f, _ in cls._fields_] == [f for f, _ in cfields[s]], s
        assert ctypes.sizeof(cls) == int(c_layout[s]), s
        for f, _ in cfields[s]:
            assert getattr(cls, f).offset == int(c_layout[f"{s}.{f}"]), (s, f)
        if ftype is None:
            continue
        body = re.search(rf"type, bind\(C\) :: {ftype}\n(.*?)end type {ftype}", ftext, flags=re.S).group(1)
        flist = []
        for line in filter(str.strip, body.replace("&\n", " ").splitlines()):
            spec, names = line.split("::")
            flist += [(n.strip().lower(), spec.strip().lower()) for n in names.split(",")]
        assert [f for f, _ in flist] == [f.lower() for f, _ in cfields[s]], s
        assert [k for _, k in flist] == [fkind[t] for _, t in cfields[s]], s


def test_python_signatures_match_the_header_prototypes():
    """The ctypes signature of every entry has the prototype's argument count,
    the same scalar types, and a pointer wherever the prototype takes one."""
    from swap_gb300 import abi

    scalar = {"int32_t": ctypes.c_int32, "int": ctypes.c_int, "uint32_t": ctypes.c_uint32,
              "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64, "double": ctypes.c_double,
              "float": ctypes.c_float, "swap_exchange_fn": abi.EXCHANGE_FN}
    pointers = (ctypes.c_void_p, ctypes.c_char_p, ctypes._Pointer)
    bad = []
    for name, (ret, types) in _header_prototypes().items():
        res, args = abi.SIGNATURES[name]
        if res is not {"int": ctypes.c_int, "const char*": ctypes.c_char_p}[ret] or len(args) != len(types):
            bad.append((name, ret, len(types), res, len(args)))
            continue
        for k, (ctype, py) in enumerate(zip(types, args)):
            ok = (isinstance(py, type) and issubclass(py, pointers)) if ctype.endswith("*") else py is scalar[ctype]
            if not ok:
                bad.append((name, k, ctype, py))
    assert not bad, bad


def test_fortran_wrappers_keep_the_reference_argument_lists():
    """The wrappers of module swap_gpu_calls carry each replaced reference
    subroutine's name and dummy arguments in order (Fortran is not case
    sensitive), against the headers recorded in tests/golden."""
    import json

    ref = json.loads((ROOT / "tests" / "golden" / "reference_interfaces.json").read_text())["subroutines"]
    text = (ROOT / "swap_gb300" / "fortran" / "swap_gpu_iface.f90").read_text()
    calls = text[text.index("module swap_gpu_calls"):]
    ours = {m.group(1).lower(): [a.strip().lower() for a in m.group(2).split(",")]
            for m in re.finditer(r"^\s*subroutine\s+(\w+)\s*\(([^)]*)\)", calls, flags=re.M)}
    assert len(ref) >= 20
    for name, sub in ref.items():
        assert ours.get(name.lower()) == [a.lower() for a in sub["args"]], (name, sub["at"], ours.get(name.lower()))


# The module state a reference subroutine reads from its modules, which the
# Python mirror takes as trailing arguments instead (the Fortran wrappers read
# it from their module): the subcycle step and count (inputs.f, gutsf.f:1776,
# 1115, 1309) and the ion step of res_chex's draws.
_MODULE_STATE = {"check_time_step": ["dtsub", "ntf"], "predict_B": ["dtsub"], "correct_B": ["dtsub"],
                 "res_chex": ["m_tstep"]}


def test_python_mirror_keeps_the_reference_argument_lists():
    """swap_gb300.hybrid.Hybrid has a method per replaced reference
    subroutine with its dummy arguments in order (np spelled np_, which
    would shadow numpy), then only the module state named above."""
    import inspect
    import json

    from swap_gb300.hybrid import Hybrid

    ref = json.loads((ROOT / "tests" / "golden" / "reference_interfaces.json").read_text())["subroutines"]
    bad = []
    for name, sub in ref.items():
        method = getattr(Hybrid, name, None)
        if method is None:
            bad.append((name, "missing"))
            continue
        got = [p.rstrip("_").lower() for p in inspect.signature(method).parameters if p != "self"]
        want = [a.lower() for a in sub["args"]] + _MODULE_STATE.get(name, [])
        if got != want:
            bad.append((name, sub["at"], want, got))
    assert not bad, bad
