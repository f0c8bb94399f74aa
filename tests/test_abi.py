"""The C-ABI library loads without a GPU and exports every entry point that
include/feng_cuda.h declares."""
import ctypes
import re

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "feng_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(fe_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "fe_cuda_solve" in names and "fe_cuda_assemble_matrices" in names
    assert len(names) > 30


def test_library_exports_every_declared_symbol(built_library):
    lib = ctypes.CDLL(str(built_library))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from feng_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_invalid_arguments_return_status_without_gpu():
    import feng_gb300 as fe
    from feng_gb300 import _lib
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.fe_mesh_generate_square(0, 0, 1, 0, 1, 0.1, 1, ctypes.byref(h)) == -3
    assert b"invalid" in lib.fe_cuda_last_error()
    assert lib.fe_mesh_read_msh(b"/nonexistent.msh", ctypes.byref(h)) == -2
    names = (ctypes.c_char_p * 1)(b"Bord")
    assert lib.fe_mesh_read_msh_groups(None, b"Domaine", names, 1, None, ctypes.byref(h)) == -3
    assert lib.fe_mesh_read_msh_groups(b"/nonexistent.msh", b"Domaine", None, 1, None, ctypes.byref(h)) == -3
    assert lib.fe_mesh_read_msh_groups(b"/nonexistent.msh", b"Domaine", names, 1, None, ctypes.byref(h)) == -2
    assert lib.fe_export_vtk(None, None, None, None, 0, None, 0, 0, b"x.vtk") == -3
