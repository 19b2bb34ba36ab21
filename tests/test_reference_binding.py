"""The reference-side bindings (hpc-mpm-code_gb300/host/reference/
gpu_solid_material_point.h, the subclass of the reference's own
SolidMaterialPointBase, and gpu_stabilized_mpm.h, the subclass of its
StabilizedMPM) compile against the reference's headers and links with libmpm_gb300.so, and the material table
it hands to the C ABI keeps every property: Mooney-Rivlin's bulk modulus
(module/solid/constitutive_model.cpp:192 reads mat_prop[2]) reaches the
context intact.  CPU only; skipped where the reference checkout is absent
(it exists only in the development container).  The reference's MPI and
PETSc headers are replaced by the oracle's single-rank stubs, and the
program links the reference's own compiled translation units
(oracle/_ref/libmpmref.so) for the base class's out-of-line members."""
import os
import subprocess

import pytest

from mpm_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MPM_REFERENCE_DIR", "/root/reference")
REFLIB = os.path.join(ROOT, "oracle", "_ref")


def _compile(tmp_path_factory, main, name):
    if not os.path.isdir(os.path.join(REF, "module", "solid")):
        pytest.skip("reference checkout absent")
    if not os.path.exists(os.path.join(REFLIB, "libmpmref.so")):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), REF], check=True)
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("binding") / name)
    cmd = ["g++", "-std=c++17", "-O1", "-w",
           "-I" + os.path.join(ROOT, "oracle", "ref_stubs"), "-I" + os.path.join(REF, "module"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "hpc-mpm-code_gb300", "host"),
           "-I" + os.path.join(ROOT, "hpc-mpm-code_gb300", "host", "reference"),
           os.path.join(ROOT, "tests", "binding", main),
           "-L" + os.path.dirname(lib), "-lmpm_gb300", "-Wl,-rpath," + os.path.dirname(lib),
           "-L" + REFLIB, "-lmpmref", "-Wl,-rpath," + REFLIB, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    return _compile(tmp_path_factory, "reference_binding_main.cpp", "reference_binding")


@pytest.fixture(scope="module")
def fluid_program(tmp_path_factory):
    return _compile(tmp_path_factory, "reference_binding_fluid_main.cpp", "reference_binding_fluid")


def test_binding_compiles_against_reference_and_keeps_material_table(program):
    out = subprocess.run([program], capture_output=True, text=True, check=True).stdout.split("\n")
    lines = {ln.split()[0] + (ln.split()[1] if ln.startswith("mat ") else ""): ln.split() for ln in out if ln}
    assert lines["nmat"][1] == "2"
    mr = lines["mat0"]
    assert int(mr[2]) == 3 and [float(v) for v in mr[3:6]] == [2.5e5, 6.25e4, 1.75e7]
    nh = lines["mat1"]
    assert int(nh[2]) == 1 and [float(v) for v in nh[3:6]] == [1.0e6, 0.3, 0.0]
    g = [float(v) for v in lines["grid"][1:]]
    assert g == [12, 0.5, 1.0e-2, 1, 2, 10, -0.25, 2.0e-2, 2, 3, 8, 0.125, 4.0e-2, 1, 2]
    c = [float(v) for v in lines["config"][1:]]
    assert c == [1.0e-5, 1.0e-12, 0.0, -1.0, -9.81, 3, 32, 1]   # APIC = 3 in MapScheme order
    assert lines["scheme"][1] == "1"   # the subclass keeps the reference's solswitch member (FLIP)


def test_fluid_binding_compiles_against_reference(fluid_program):
    """The stabilized-fluid binding (host/reference/gpu_stabilized_mpm.h, a
    subclass of the reference's StabilizedMPM) compiles against the reference's
    headers and hands the C ABI the grid globals, the object's fluid constants
    and Newmark coefficients, gravity, facl and mtol unchanged."""
    out = subprocess.run([fluid_program], capture_output=True, text=True, check=True).stdout.split("\n")
    lines = {ln.split()[0]: ln.split() for ln in out if ln}
    g = [float(v) for v in lines["grid"][1:]]
    assert g == [6, 0.0, 1.0e-2, 1, 2, 5, 0.5, 2.0e-2, 1, 2, 4, -1.0, 1.0e-2, 1, 2]
    p = [float(v) for v in lines["params"][1:]]
    assert p == [1000.0, 1.0e-3, 2.0e-3, 0.25, 0.5, 0.0, 0.0, -9.8, 0.75, 1.0e-12]
    assert lines["scheme"][1] == "1"   # FLIP in MapScheme order
