"""The script front end (femmd_old_gb300/frontend/md_js.cpp): the
reference's System object, file helpers and tables over the C ABI
(interface.cpp:86-756).  It is built only where Duktape's sources exist (the
reference vendors them); these tests skip elsewhere.  Without a GPU a script
runs through every host-side call and stops at the first device call with
the library's error; the reference's own test.js runs unmodified that far."""
import json
import os
import subprocess

import numpy as np
import pytest

import femmd_old_gb300 as F
from femmd_old_gb300 import build as B
from femmd_old_gb300 import scene as S

BIN = B.FRONTEND_BIN
pytestmark = pytest.mark.skipif(not os.path.exists(BIN), reason="script front end not built (no Duktape sources)")


def run_script(tmp_path, text, name="script.js"):
    path = tmp_path / name
    path.write_text(text)
    r = subprocess.run([BIN, str(path)], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    return r.returncode, r.stdout


def tagged(out, tag):
    return [line[len(tag) + 1:] for line in out.splitlines() if line.startswith(tag + " ")]


def test_setup_calls_files_and_getters(tmp_path):
    rc, out = run_script(tmp_path, """
function mdmain() {
    System.DEV(DEV.CPU);
    System.init(20, 16);
    System.PBC(PBCTYPE.XPBC);
    System.set_dt(0.002);
    System.set_numTypes(1);
    System.set_kBond(50);
    System.set_youngs_modulus(30);
    System.set_pair_potential(new Float64Array([1.0]), new Float64Array([2.5]), new Float64Array([0.0]));
    System.add_particle(1.0, 2.0, 0.0, 0.0, 1.0, 1.0, 0);
    System.add_particle(3.0, 2.0, 0.5, 0.0, 1.0, 1.0, 0);
    write_to_file("a.txt", "1 2 3\\n");
    append_to_file("a.txt", "4 5\\n");
    make_dir("sub");
    change_dir("sub");
    write_to_file("b.txt", "0.5 1.5\\n");
    var f = read_file("b.txt", FILECONTENT.FLOAT);
    change_dir("..");
    var ints = read_file("a.txt", FILECONTENT.INT);
    print("INTS", ints.length, ints[0], ints[4]);
    print("FLOATS", f.length, f[1]);
    print("TEXT", JSON.stringify(read_file("a.txt", FILECONTENT.TEXT)));
    print("INFO", JSON.stringify(System.info()));
    print("BOX", JSON.stringify(System.get_box()));
    print("DT", System.get_dt());
    System.set_box(24, 18);
    print("BOX2", JSON.stringify(System.get_box()));
}
""")
    assert rc == 0, out
    assert tagged(out, "INTS") == ["5 1 5"]
    assert tagged(out, "FLOATS") == ["2 1.5"]
    assert json.loads(tagged(out, "TEXT")[0]) == "1 2 3\n4 5\n"
    info = json.loads(tagged(out, "INFO")[0])
    assert info["N"] == 2 and info["nelastomers"] == 0 and info["kBonds"] == 50 and info["E"] == 30
    assert info["box"] == {"x": 20, "y": 16}
    assert json.loads(tagged(out, "BOX2")[0]) == {"x": 24, "y": 18}
    assert abs(float(tagged(out, "DT")[0]) - 0.002) < 1e-9
    assert (tmp_path / "sub" / "b.txt").exists()


def test_elastomers_match_the_library_called_directly(tmp_path):
    verts, tris = S.hex_disk_mesh(1.0, 2)
    np.savetxt(tmp_path / "v.txt", np.asarray(verts, np.float32).reshape(-1, 2), fmt="%.8g")
    np.savetxt(tmp_path / "t.txt", np.asarray(tris, np.int32).reshape(-1, 3), fmt="%d")
    rc, out = run_script(tmp_path, """
function mdmain() {
    System.init(30, 30);
    System.set_kBond(100);
    var v = read_file("v.txt", FILECONTENT.FLOAT);
    var t = read_file("t.txt", FILECONTENT.INT);
    for (var k = 0; k < 4; k++)
        System.add_elastomer(v, t, 5 + 6 * k, 10, 0, 0, 1.0, 1.0, true);
    System.add_particle(25.0, 25.0, 0.0, 0.0, 1.0, 1.0, 0);
    print("INFO", JSON.stringify(System.info()));
}
""")
    assert rc == 0, out
    info = json.loads(tagged(out, "INFO")[0])
    s = F.System(0)
    s.init(30, 30)
    s.set_kBond(100)
    vf = np.loadtxt(tmp_path / "v.txt", dtype=np.float32).ravel()
    ti = np.loadtxt(tmp_path / "t.txt", dtype=np.int32).ravel()
    for k in range(4):
        s.add_elastomer(vf, ti, 5 + 6 * k, 10, 0, 0, 1.0, 1.0, True)
    s.add_particle(25.0, 25.0, 0.0, 0.0, 1.0, 1.0, 0)
    direct = s.info()
    assert info["nelastomers"] == 4 and direct["nelastomers"] == 4
    for key in ("N", "nbonds", "ntrigs", "kBonds"):
        assert info[key] == direct[key], key
    assert info["ntrigs"] == s.counts()["triangles"] > 0


def test_library_errors_end_mdmain(tmp_path):
    rc, out = run_script(tmp_path, """
function mdmain() {
    System.init(10, 10);
    System.set_pair_potential(new Float64Array([1.0]), new Float64Array([2.5]), new Float64Array([0.0]));
    System.add_particle(1.0, 1.0, 0.0, 0.0, 1.0, 1.0, 0);
    System.add_particle(7.0, 1.0, 0.0, 0.0, 1.0, 1.0, 0);
    System.init_neighbor_list();
    System.run(10);
    print("NOT REACHED");
}
""")
    # without a GPU run() fails; with one it would have returned
    assert "NOT REACHED" not in out or rc == 0
    if rc != 0:
        assert rc == 2
        assert any(line.startswith("Error: ") and "run:" in line for line in out.splitlines()), out
    # a call out of order fails the same way, with the library's message
    rc2, out2 = run_script(tmp_path, """
function mdmain() {
    System.add_particle(1.0, 1.0, 0.0, 0.0, 1.0, 1.0, 0);
    print("NOT REACHED");
}
""", name="order.js")
    assert rc2 == 2 and "NOT REACHED" not in out2
    assert "Error: Error: add_particle: init(Lx, Ly) has not been called" in out2


def test_reference_script_runs_unmodified_to_the_device(tmp_path):
    # the reference's own src/test.js, shipped beside the Duktape sources the
    # front end was built from; its two mesh files are not in the reference,
    # so a hexagonal disk mesh stands in for them
    src = open(BIN + ".src").read().strip()
    script = os.path.join(src, "test.js")
    if not os.path.exists(script):
        pytest.skip("the reference's test.js is not beside the Duktape sources")
    verts, tris = S.hex_disk_mesh(1.0, 2)
    np.savetxt(tmp_path / "squareVertices5v.txt", np.asarray(verts, np.float32).reshape(-1, 2), fmt="%.8g")
    np.savetxt(tmp_path / "squareTriangles5v.txt", np.asarray(tris, np.int32).reshape(-1, 3), fmt="%d")
    r = subprocess.run([BIN, script], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    out = r.stdout
    # its runOne: 8 x 8 cells, two elastomers each, then System.info() as JSON
    start = out.index("system info")
    info, _ = json.JSONDecoder().raw_decode(out, out.index("{", start))
    nv = len(np.asarray(verts).reshape(-1, 2))
    assert info["nelastomers"] == 128 and info["N"] == 128 * nv
    assert info["ntrigs"] == 128 * len(np.asarray(tris).reshape(-1, 3)) and info["E"] == 50
    # every call before System.allocate_cuda went through; without a GPU that one fails
    if r.returncode != 0:
        assert "Error: Error: allocate_cuda:" in out
