"""C ABI: the library builds, loads and exports every entry point include/mpasg.h declares,
and the ctypes struct layouts match the header field for field (no GPU needed)."""

import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = (ROOT / "include" / "mpasg.h").read_text()


def _lib_path():
    from mpas_dycore_pytorch_gb300.build import build
    try:
        return build()
    except RuntimeError as exc:  # no nvcc on this machine
        pytest.skip(str(exc))


def _declared_functions():
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char \*)\s*(mpasg_\w+)\s*\(", HEADER, re.M)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_lib_path()))
    names = _declared_functions()
    assert len(names) >= 17
    for name in names:
        assert hasattr(lib, name), name
    from mpas_dycore_pytorch_gb300 import _lib
    assert sorted(_lib.EXPORTS) == names


def _struct_fields(name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), HEADER, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        parts = decl.replace("\n", " ")
        names = re.sub(r"^(const\s+)?(int32_t|double|float)\s*", "", parts)
        for n in names.split(","):
            out.append(n.replace("*", "").strip())
    return out


@pytest.mark.parametrize("cname,pyname", [("mpasg_mesh", "MeshStruct"), ("mpasg_config", "ConfigStruct"),
                                          ("mpasg_fields", "FieldsStruct")])
def test_ctypes_layout_matches_header(cname, pyname):
    from mpas_dycore_pytorch_gb300 import _lib
    py = [f[0] for f in getattr(_lib, pyname)._fields_]
    assert _struct_fields(cname) == py


def test_abi_version_and_build_info():
    from mpas_dycore_pytorch_gb300 import _lib
    lib = ctypes.CDLL(str(_lib_path()))
    lib.mpasg_build_info.restype = ctypes.c_char_p
    assert lib.mpasg_abi_version() == _lib.ABI_VERSION
    assert b"sm_103a" in lib.mpasg_build_info()
