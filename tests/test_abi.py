"""The drop-in boundary: libbfm.so loads and exports every declared symbol."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include" / "bfm").glob("*.h"))


def declared_functions(path: Path) -> set[str]:
    src = re.sub(r"/\*.*?\*/", "", path.read_text(), flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    names = set()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(bfm_\w+)\s*\(", src, flags=re.M):
        if "typedef" in src[max(0, m.start() - 0):m.end()].split("\n")[-1]:
            continue
        names.add(m.group(1))
    return names


def test_headers_declare_the_reference_api():
    names = set().union(*(declared_functions(h) for h in HEADERS))
    # a sample of the reference entry points (libbfm/src/bfm/*.h) that must stay
    for n in ["bfm_sim_run", "bfm_system_create_planar_stress", "bfm_perm_rcm", "bfm_matrix_solve",
              "bfm_mesh_read_lepl1110", "bfm_ez_lepl1110_create", "bfm_condition_create", "bfm_state_create"]:
        assert n in names
    assert len(names) > 80


def test_library_exports_every_declared_symbol(libbfm_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(libbfm_path)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = set()
    for h in HEADERS:
        missing |= declared_functions(h) - exported
    assert not missing, f"not exported: {sorted(missing)}"


def test_entry_points_carry_nvtx_ranges(libbfm_path):
    """The entry points and set-up phases push NVTX ranges named after them
    (header-only NVTX: nothing of it is exported)."""
    data = Path(libbfm_path).read_bytes()
    for name in (b"bfm_sim_run", b"bfm_gpu_problem_assemble", b"bfm_gpu_problem_solve", b"bfm_gpu_problem_step_parts",
                 b"bfm_gpu_mpnn_forward", b"color_nodes", b"coarse_setup", b"autotune_lpr"):
        assert name + b"\0" in data, name
    out = subprocess.run(["nm", "-D", "--defined-only", str(libbfm_path)], capture_output=True, text=True,
                         check=True).stdout
    assert "nvtx" not in out.lower()


def test_library_loads_and_binds(libbfm):
    assert libbfm.bfm_gpu_device_count() >= 0
    s = __import__("bfm_gb300.abi", fromlist=["x"]).bfm_state_t()
    assert libbfm.bfm_state_create(C.byref(s)) == 0


def test_struct_sizes_match_the_c_abi(tmp_path):
    """sizeof/offsetof of every public struct, compiled from include/bfm vs the ctypes mirror."""
    from bfm_gb300 import abi
    structs = ["bfm_state_t", "bfm_vec_t", "bfm_edge_t", "bfm_domain_t", "bfm_mesh_t", "bfm_material_t",
               "bfm_shape_t", "bfm_rule_t", "bfm_force_t", "bfm_condition_t", "bfm_obj_t", "bfm_instance_t",
               "bfm_sim_t", "bfm_matrix_t", "bfm_perm_t", "bfm_system_t", "bfm_ez_lepl1110_t"]
    prog = "#include <stdio.h>\n#include <bfm/ez.h>\n#include <bfm/system.h>\nint main(void){\n"
    prog += "".join(f'printf("%zu\\n", sizeof({s}));\n' for s in structs) + "return 0;}\n"
    (tmp_path / "s.c").write_text(prog)
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(tmp_path / "s.c"), "-o", str(tmp_path / "s")], check=True)
    sizes = [int(x) for x in subprocess.run([str(tmp_path / "s")], capture_output=True, text=True).stdout.split()]
    for s, n in zip(structs, sizes):
        assert C.sizeof(getattr(abi, s)) == n, s
