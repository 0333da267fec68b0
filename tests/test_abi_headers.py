"""The drop-in boundary from C and C++: include/rtbvh.h compiled as C11 and
include/rtbvh.hpp (the reference's cbindgen C++ form: namespace rtbvh,
enum class types, include guard RTBVH_HPP; rtbvh_ffi/build.rs:15-45) as
C++17, both linked against librtbvh_rs.so, the file name the reference's
C/C++ users link (rtbvh_ffi/Cargo.toml).

The programs in tests/abi/ static_assert every struct's size and field
offsets (rtbvh_ffi/src/lib.rs:855-866), make the argument-error calls of
create_delete (:868-904) without a GPU, and with a GPU run create_delete
and the t == 1 quad of the intersect test (:945-1019)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
ABI = os.path.join(ROOT, "tests", "abi")


def _declared(path):
    """Function names declared in a header (a return type, a name, an
    opening parenthesis at the start of a line)."""
    text = open(path).read()
    return set(re.findall(r"^(?:const )?[A-Za-z_][A-Za-z0-9_]* \*?([A-Za-z_][A-Za-z0-9_]*)\(", text, re.M))


@pytest.fixture(scope="module")
def programs(lib, tmp_path_factory):
    from rtbvh_gb300 import build as libbuild
    out = tmp_path_factory.mktemp("abi")
    libdir = os.path.dirname(libbuild.ALIAS)
    c_exe, cpp_exe = str(out / "abi_c"), str(out / "abi_cpp")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", INC, os.path.join(ABI, "abi_check.c"),
                    "-L", libdir, "-lrtbvh_rs", "-lm", "-o", c_exe], check=True)
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", INC,
                    os.path.join(ABI, "abi_check.cpp"), "-L", libdir, "-lrtbvh_rs", "-o", cpp_exe], check=True)
    env = dict(os.environ, LD_LIBRARY_PATH=libdir + os.pathsep + os.environ.get("LD_LIBRARY_PATH", ""))
    return c_exe, cpp_exe, env


def test_headers_declare_the_same_functions_and_the_library_exports_them(lib):
    c_names = _declared(os.path.join(INC, "rtbvh.h"))
    cpp_names = _declared(os.path.join(INC, "rtbvh.hpp"))
    ref = {"create_spatial_Bvh", "create_bvh", "create_mbvh", "refit", "intersect", "intersect_packet",
           "intersect_mbvh", "intersect_mbvh_packet", "free_bvh", "free_mbvh"}
    assert ref <= c_names
    assert c_names == cpp_names, (c_names ^ cpp_names)
    for name in sorted(c_names):
        assert hasattr(lib, name), f"{name} not exported"


def test_c_and_cpp_programs_compile_link_and_reject_bad_arguments(programs):
    c_exe, cpp_exe, env = programs
    for exe in (c_exe, cpp_exe):
        r = subprocess.run([exe, "args"], env=env, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_c_and_cpp_programs_build_and_hit_the_quad_at_t_1(programs):
    c_exe, cpp_exe, env = programs
    for exe in (c_exe, cpp_exe):
        r = subprocess.run([exe, "gpu"], env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
