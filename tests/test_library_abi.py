"""The C-ABI libraries load and export every function their headers declare,
and OSQP's unmodified C core links against the algebra library (CPU only)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO, reference_dir

INCLUDE = os.path.join(REPO, "include")
LIBDIR = os.path.join(REPO, "osqp_gb300", "lib")

HEADERS = {
    "osqp_gb300.h": ["libosqp_gb300.so", "libosqp_gb300_f64.so"],
    "osqp_gb300_ext.h": ["libosqp_gb300.so", "libosqp_gb300_f64.so"],
    "osqp_gb300_algebra.h": ["libosqp_gb300_algebra.so", "libosqp_gb300_algebra_f64.so"],
}


@pytest.fixture(scope="module")
def libs():
    from osqp_gb300.build import build
    return build()


def declared_functions(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = set()
    for m in re.finditer(r"\b((?:osqp|OSQP)\w*)\s*\(", text):
        name = m.group(1)
        if text[m.end():m.end() + 1] == "*" or name in ("OSQPInt", "OSQPFloat") or name.isupper():
            continue   # function-pointer fields and type names, not functions
        names.add(name)
    return sorted(names)


@pytest.mark.parametrize("header", sorted(HEADERS))
def test_headers_are_exported(libs, header):
    names = declared_functions(header)
    assert len(names) > 5
    for lib in HEADERS[header]:
        path = os.path.join(LIBDIR, lib)
        handle = ctypes.CDLL(path)   # loads without a GPU: no device work at load time
        missing = [n for n in names if not hasattr(handle, n)]
        assert not missing, (lib, missing)


def test_public_api_matches_reference_symbol_set(libs):
    """Every function of OSQP's public header (include/public/osqp_api_functions.h)
    has a definition in the GB300 library."""
    expected = ["osqp_capabilities", "osqp_version", "osqp_error_message", "osqp_get_dimensions",
                "osqp_setup", "osqp_solve", "osqp_get_solution", "osqp_cleanup", "osqp_warm_start",
                "osqp_cold_start", "osqp_update_data_vec", "osqp_update_data_mat", "osqp_set_default_settings",
                "osqp_update_settings", "osqp_update_rho", "osqp_adjoint_derivative_compute",
                "osqp_adjoint_derivative_get_mat", "osqp_adjoint_derivative_get_vec",
                "osqp_set_default_codegen_defines", "osqp_codegen", "OSQPCscMatrix_new", "OSQPCscMatrix_free",
                "OSQPCscMatrix_zeros", "OSQPCscMatrix_identity", "OSQPCscMatrix_diag_scalar",
                "OSQPCscMatrix_diag_vec", "OSQPCscMatrix_set_data", "OSQPSettings_new", "OSQPSettings_free",
                "OSQPCodegenDefines_new", "OSQPCodegenDefines_free"]
    handle = ctypes.CDLL(os.path.join(LIBDIR, "libosqp_gb300.so"))
    assert [n for n in expected if not hasattr(handle, n)] == []


def test_host_only_entry_points_without_gpu(libs):
    """Settings defaults and CSC helpers work on a machine without a GPU."""
    from osqp_gb300.api import Library
    for name, bits in (("libosqp_gb300.so", 32), ("libosqp_gb300_f64.so", 64)):
        L = Library(os.path.join(LIBDIR, name), bits)
        st = L.default_settings()
        # the CUDA-build defaults (include/public/osqp_api_constants.h:111-178)
        assert st.rho_is_vec == 0 and st.check_termination == 5 and abs(st.adaptive_rho_tolerance - 2.0) < 1e-6
        assert st.linsys_solver == 2 and st.max_iter == 4000 and st.scaling == 10
        assert st.check_dualgap == (0 if bits == 32 else 1)
        L.lib.osqp_error_message.restype = ctypes.c_char_p
        assert b"validation" in L.lib.osqp_error_message(1)


@pytest.mark.skipif(not reference_dir(), reason="reference sources not present")
def test_reference_core_links_against_gb300_algebra(libs):
    """OSQP's own C core (src/*.c, unmodified) links against libosqp_gb300_algebra
    with --no-undefined: the algebra / linear-system boundary is complete."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "dropin"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    for so in ("libosqp_core_on_gb300.so", "libosqp_core_on_gb300_f64.so"):
        path = os.path.join(REPO, "oracle", "_ref", so)
        out = subprocess.run(["nm", "-D", "--undefined-only", path], capture_output=True, text=True).stdout
        undefined = {l.split()[-1] for l in out.splitlines() if l.strip()}
        ours = {s for s in undefined if s.startswith(("OSQPVector", "OSQPMatrix", "osqp_algebra"))}
        handle = ctypes.CDLL(os.path.join(LIBDIR, "libosqp_gb300_algebra.so" if "f64" not in so
                                          else "libosqp_gb300_algebra_f64.so"))
        assert ours and all(hasattr(handle, s) for s in ours)
