"""CPU checks of the drop-in boundary: the C-ABI library loads and exports
every function include/gbferm.h declares; host-side parameter handling."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gbferm.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\**\s*\**(gbf_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_reference_boundary():
    names = declared_functions()
    # cgpt create/update/set_mass/delete/apply_fermion_operator (operators.cc:34-133)
    for n in ["gbf_create", "gbf_update_gauge", "gbf_set_mass", "gbf_delete", "gbf_apply",
              "gbf_solve_eo2ne_cg", "gbf_norm2", "gbf_inner", "gbf_axpby", "gbf_convert", "gbf_last_error"]:
        assert n in names, n


def test_library_loads_and_exports_every_symbol():
    from gpt_gb300 import _lib

    L = _lib.load()
    for n in declared_functions():
        assert hasattr(L, n), f"{n} declared in include/gbferm.h but not exported"
    # no GPU work: the error channel works without a device
    assert isinstance(L.gbf_last_error(), bytes)


def test_create_rejects_bad_arguments_without_touching_the_gpu():
    from gpt_gb300 import _lib

    L = _lib.load()
    p = _lib.gbf_params()
    for i, d in enumerate([4, 4, 4, 3]):  # odd extent
        p.dims[i] = d
    p.Ls, p.n_rhs = 1, 1
    h = ctypes.c_void_p()
    rc = L.gbf_create(b"wilson_clover", 0, ctypes.byref(p), ctypes.byref(h))
    assert rc == 1 and b"even" in L.gbf_last_error()
    p.dims[3] = 4
    rc = L.gbf_create(b"staggered", 0, ctypes.byref(p), ctypes.byref(h))
    assert rc == 5
    p.n_rhs = 17
    rc = L.gbf_create(b"wilson_clover", 0, ctypes.byref(p), ctypes.byref(h))
    assert rc == 1 and b"n_rhs" in L.gbf_last_error()


def test_structs_match_the_c_compiler(tmp_path):
    """ctypes mirrors of the header structs have the sizes and offsets gcc gives."""
    import subprocess

    from gpt_gb300 import _lib

    prog = tmp_path / "sz.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "gbferm.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(gbf_params), sizeof(gbf_cg_params),"
        " sizeof(gbf_cg_result), offsetof(gbf_params, boundary_phases), offsetof(gbf_params, reconstruct),"
        " offsetof(gbf_cg_result, kernel_launches)); return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = [ctypes.sizeof(_lib.gbf_params), ctypes.sizeof(_lib.gbf_cg_params), ctypes.sizeof(_lib.gbf_cg_result),
            _lib.gbf_params.boundary_phases.offset, _lib.gbf_params.reconstruct.offset,
            _lib.gbf_cg_result.kernel_launches.offset]
    assert got == want


def test_wilson_clover_parameter_handling(monkeypatch):
    from gpt_gb300.qcd import fermion

    with pytest.raises(ValueError):
        fermion.wilson_clover(None, {"mass": 0.1, "cF": 1.3, "boundary_phases": [1, 1, 1, -1]})
    # mobius with per-slice omega is the zmobius operator
    seen = {}
    monkeypatch.setattr(fermion, "zmobius", lambda U, p: seen.setdefault("p", p))
    fermion.mobius(None, {"omega": [1.0, 0.5], "mass": 0.1, "b": 1.0, "c": 0.0, "M5": 1.8})
    assert seen["p"]["omega"] == [1.0, 0.5]
