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
