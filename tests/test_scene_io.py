"""The reference's on-disk formats through the C++ host layer
(hpc-mpm-code_gb300/host/scene_io.cpp, driven by scene_tool).

The fixtures in tests/golden/io/ come from the reference itself
(tests/golden/make_golden.py --io): the grid and particle decks as its own
readers (InputParaGriddata, BCInput, InputPointData) parsed them, and the
restarts its RestartOutput wrote after 10 steps of a TPIC and an APIC block.
"""
import os
import subprocess

import numpy as np
import pytest

from helpers import rel_l2
from mpm_gb300 import build

IO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io")


def _golden():
    return np.load(os.path.join(IO, "io.npz"))


def _tool():
    build.build_host()
    return build.SCENE_TOOL


def _parse_tool_output(text):
    out = {}
    for line in text.strip().splitlines():
        name, *vals = line.split()
        out[name] = np.array([float(v) for v in vals])
    return out


def test_decks_parse_like_the_reference():
    """Every value InputParaGriddata, the three BCInput lists and
    InputPointData read from the same decks, exactly."""
    g = _golden()
    r = subprocess.run([_tool(), "parse", os.path.join(IO, "grid0.txt"), os.path.join(IO, "point0.txt")],
                       capture_output=True, text=True, check=True)
    o = _parse_tool_output(r.stdout)
    assert np.array_equal(o["ints"].astype(np.int64), g["parsed_ints"].astype(np.int64))
    assert np.array_equal(o["dbl"], g["parsed_dbl"])
    for k in range(3):
        assert np.array_equal(o[f"bc{k}_nodes"], g[f"parsed_bc{k}_nodes"])
        assert np.array_equal(o[f"bc{k}_vals"], g[f"parsed_bc{k}_vals"])
    assert np.array_equal(o["coord"].reshape(-1, 3), g["parsed_coord"])
    for k in ("id", "matid", "surf", "mass", "vol0"):
        assert np.array_equal(o[k], g[f"parsed_{k}"]), k


def test_tpic_restart_round_trip_is_byte_identical(tmp_path):
    """RestartInput then RestartOutput of a restart the reference wrote
    reproduces the file byte for byte."""
    src = os.path.join(IO, "restart_tpic0_re.txt")
    dst = str(tmp_path / "rt.txt")
    subprocess.run([_tool(), "copy-restart", "TPIC", src, dst], check=True)
    with open(src, "rb") as a, open(dst, "rb") as b:
        assert a.read() == b.read()


def _restart_sections(path, n):
    """The restart's lines after the header: coord, records, vel, accel,
    stress, F, then the scheme's matrices, each n lines."""
    with open(path) as f:
        lines = f.read().splitlines()
    assert int(lines[0].split()[0]) == n
    body = lines[1:]
    return [np.array([[float(v) for v in ln.split()] for ln in body[k * n:(k + 1) * n]]) for k in range(len(body) // n)]


def test_apic_restart_keeps_the_affine_product(tmp_path):
    """An APIC restart written here carries vel_Bmat . inv_Dmat of the
    reference's restart as vel_Bmat (with inv_Dmat the identity): the
    product the transfers use, to the file's 6 significant digits; every
    other section is byte-identical, and a second round trip is too."""
    src = os.path.join(IO, "restart_apic0_re.txt")
    a, b = str(tmp_path / "a.txt"), str(tmp_path / "b.txt")
    subprocess.run([_tool(), "copy-restart", "APIC", src, a], check=True)
    subprocess.run([_tool(), "copy-restart", "APIC", a, b], check=True)
    with open(a, "rb") as fa, open(b, "rb") as fb:
        assert fa.read() == fb.read()
    n = 512
    ref, ours = _restart_sections(src, n), _restart_sections(a, n)
    assert len(ref) == len(ours) == 9
    for k in range(6):
        assert np.array_equal(ref[k], ours[k]), k
    prod = np.einsum("pik,pkj->pij", ref[6].reshape(n, 3, 3), ref[8].reshape(n, 3, 3)).reshape(n, 9)
    assert np.allclose(ours[6], prod, rtol=1e-6, atol=1e-6 * np.abs(prod).max())
    assert np.array_equal(ours[7], np.zeros((n, 9)))
    assert np.array_equal(ours[8], np.tile(np.eye(3).ravel(), (n, 1)))


def test_multi_rank_grid_deck_is_refused(tmp_path):
    """A rank with overlap neighbours (isb != 0) needs the halo exchange the
    single-GPU path does not have: the reader refuses it."""
    lines = open(os.path.join(IO, "grid0.txt")).read().splitlines()
    k = next(i for i, ln in enumerate(lines) if "overlapped ranks" in ln)
    lines[k] = "1     --- overlapped ranks ---"
    bad = tmp_path / "grid0.txt"
    bad.write_text("\n".join(lines) + "\n")
    r = subprocess.run([_tool(), "parse", str(bad), os.path.join(IO, "point0.txt")], capture_output=True, text=True)
    assert r.returncode == 2 and "isb" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_restart_continuation_matches_reference(precision, tmp_path):
    """The decks plus the reference's APIC restart, run 10 steps on the GPU
    through the host layer, against the reference's own continuation of the
    same restart: FP64 1e-10 (affine matrix included); FP32 1e-6 on x,
    1e-4 on v, 1e-3 on the affine matrix."""
    g = _golden()
    prefix = str(tmp_path / "out")
    subprocess.run([_tool(), "run", os.path.join(IO, "para.txt"), os.path.join(IO, "grid0.txt"),
                    os.path.join(IO, "restart_apic0_re.txt"), str(int(g["cont_nsteps"])), str(precision), prefix],
                   check=True, capture_output=True, text=True)
    n = g["cont_x"].shape[0]
    raw = np.fromfile(prefix + ".bin", dtype=np.float64)
    sizes = [3, 3, 9, 6, 1, 9]
    parts, o = [], 0
    for w in sizes:
        parts.append(raw[o:o + w * n])
        o += w * n
    x, v, F, sig, vol, aff = parts
    e = {"x": rel_l2(x, g["cont_x"].ravel()), "v": rel_l2(v, g["cont_v"].ravel()),
         "F": rel_l2(F, g["cont_F"].ravel()), "sigma": rel_l2(sig, g["cont_sigma"].ravel()),
         "vol": rel_l2(vol, g["cont_vol"]), "affine": rel_l2(aff, g["cont_affine"].ravel())}
    assert os.path.exists(prefix + "0_re.txt")
    if precision == 64:
        assert max(e.values()) <= 1e-10, e
    else:
        assert e["x"] <= 1e-6 and e["v"] <= 1e-4 and e["affine"] <= 1e-3, e
