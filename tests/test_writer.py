"""Output writers of the host library (include/sph_host.h: sph_write_output, sph_write_mesh)
against the file layout of OutputRes / OutputMesh (code/3_SPH_material_2018.f90:2707-3010)."""
import numpy as np
import pytest

import cases


def _f16_8(v):
    s = "%16.8f" % v
    return "*" * 16 if len(s) > 16 else s


def _fields(prob):
    s = prob.state()
    bc = prob.bc_or_not.copy()
    bc[: prob.nnode: 7] = 2  # mark some nodes as free-surface nodes
    rng = np.random.default_rng(3)
    s["stress"] = rng.uniform(-3e5, 3e5, s["stress"].size)
    s["vel"] = rng.uniform(-1, 1, s["vel"].size)
    s["intvars1"] = rng.uniform(0, 1e-2, s["intvars1"].size)
    return dict(x=s["x"], vel=s["vel"], stress=s["stress"], rho=s["rho"],
                intvars1=s["intvars1"], displ=rng.uniform(-1e-3, 1e-3, 2 * prob.nnode),
                bc_or_not=bc)


def test_output_flags_default_and_custom():
    p = cases.bui_like(width=0.5, height=0.3, dx=0.1)
    assert p.output_flags() == dict(sxx=1, syy=1, sxy=1, szz=1, vx=1, vy=1, strain=1, rho=0,
                                    sml=0, disp=0)


def test_nodes_and_stress_points_files(tmp_path):
    p = cases.bui_like(width=0.5, height=0.3, dx=0.1)
    f = _fields(p)
    p.write_output(tmp_path, 12, 0.25, f, hsml=p.hsml)
    nodes = (tmp_path / "nodes.csv.000012").read_text().split("\n")
    assert nodes[0] == "x-coord,,y-coord,x-vel,y-vel,sxx,syy,sxy,szz,strain  "
    assert len(nodes) == p.nnode + 2 and nodes[-1] == ""
    for i in range(p.nnode):
        want = ",".join([_f16_8(f["x"][2 * i]), _f16_8(f["x"][2 * i + 1]),
                         _f16_8(f["vel"][2 * i]), _f16_8(f["vel"][2 * i + 1])] +
                        [_f16_8(f["stress"][4 * i + k]) for k in range(4)] +
                        [_f16_8(f["intvars1"][i])]) + "  "
        assert nodes[1 + i] == want
    sp = (tmp_path / "stress_points.csv.000012").read_text().split("\n")
    assert sp[0] == "x-coord,y-coord,x-vel,y-vel,sxx,syy,sxy,szz,strain,  "
    assert len(sp) == p.nstress + 2
    for i in range(p.nnode, p.ntotal):
        want = "".join(_f16_8(v) + "," for v in
                       [f["x"][2 * i], f["x"][2 * i + 1], f["vel"][2 * i], f["vel"][2 * i + 1]] +
                       [f["stress"][4 * i + k] for k in range(4)] + [f["intvars1"][i]]) + "  "
        assert sp[1 + i - p.nnode] == want


def test_surface_points_file(tmp_path):
    p = cases.bui_like(width=0.5, height=0.3, dx=0.1)
    f = _fields(p)
    p.write_output(tmp_path, 0, 0.0, f)
    lines = (tmp_path / "surface_points.csv.000000").read_text().strip("\n").split("\n")
    assert lines[0].split() == ["x-coord,y-coord,"]
    on = np.nonzero(f["bc_or_not"][: p.nnode] == 2)[0]
    assert len(lines) == 1 + len(on)
    got = np.array([[float(t) for t in ln.replace(",", " ").split()] for ln in lines[1:]])
    np.testing.assert_array_equal(got[:, 0], f["x"][2 * on])
    np.testing.assert_array_equal(got[:, 1], f["x"][2 * on + 1])


def test_wide_values_are_starred(tmp_path):
    p = cases.bui_like(width=0.5, height=0.3, dx=0.1)
    f = _fields(p)
    f["stress"][0] = -2.5e7  # 17 characters in F16.8: the field is filled with asterisks
    p.write_output(tmp_path, 1, 0.0, f)
    row = (tmp_path / "nodes.csv.000001").read_text().split("\n")[1].split(",")
    assert row[4] == "*" * 16


def _gid_blocks(text):
    """{(result name, time): [(id, values...)]} of a GiD results file."""
    out, cur = {}, None
    for ln in text.split("\n"):
        t = ln.strip()
        if t.startswith("Result"):
            name = t.split('"')[1]
            time = float(t.split('"')[4].split()[0])
            cur = out.setdefault((name, time), [])
        elif t.startswith("End Values"):
            cur = None
        elif cur is not None and t and not t.startswith("Values"):
            cur.append([float(v) for v in t.split()])
    return out


def test_gid_results_and_mesh(tmp_path):
    p = cases.bui_like(width=0.5, height=0.3, dx=0.1)
    p.write_mesh(tmp_path)
    f = _fields(p)
    p.write_output(tmp_path, 1, 0.125, f)
    p.write_output(tmp_path, 2, 0.25, f)
    res = (tmp_path / (p.name + ".post.res")).read_text()
    assert res.count("GiD Post Results File 1.0") == 1
    blocks = _gid_blocks(res)
    names = sorted({k[0] for k in blocks})
    assert names == ["disp", "plastic strain", "sigmaxx", "sigmaxy", "sigmayy", "vel"]
    nn = p.nnode
    for t in (0.125, 0.25):
        vel = np.array(blocks[("vel", t)])
        assert vel.shape == (nn, 4)
        np.testing.assert_array_equal(vel[:, 0], np.arange(1, nn + 1))
        np.testing.assert_array_equal(vel[:, 1], f["vel"][0:2 * nn:2])
        ux, uy = f["vel"][0:2 * nn:2], f["vel"][1:2 * nn:2]
        np.testing.assert_array_equal(vel[:, 3], np.sqrt(ux ** 2 + uy ** 2))  # umod
        sxy = np.array(blocks[("sigmaxy", t)])
        np.testing.assert_array_equal(sxy[:, 1], f["stress"][2:4 * nn:4])
        disp = np.array(blocks[("disp", t)])
        # positions are updated in this problem: displacement = x - x00
        np.testing.assert_array_equal(disp[:, 1], f["x"][0:2 * nn:2] - p.x00[0:2 * nn:2])
    msh = (tmp_path / (p.name + ".post.msh")).read_text().split("\n")
    i0 = msh.index("  Elements")
    elems = [list(map(int, ln.split())) for ln in msh[i0 + 1:] if ln.strip()
             and not ln.strip().startswith("End")]
    ndivx, ndivy = int(0.5 / 0.1 + 1.0), int(0.3 / 0.1 + 1.0)  # Read_2DMesh: lx/dx + 1
    assert len(elems) == (ndivx - 1) * (ndivy - 1)
    # first cell of the second lattice column: nodes ndivy+2, 2, 1, ndivy+1
    assert elems[0] == [1, ndivy + 2, 2, 1, ndivy + 1, 1]


@pytest.mark.parametrize("flags", ["1 0 1 0 0 1 1 1 1 1", "0 0 0 0 0 0 0 0 0 0"])
def test_custom_output_selection(tmp_path, flags):
    p = cases.bui_like(width=0.5, height=0.3, dx=0.1, output_flags=flags)
    want = dict(zip(p.OUTPUT_FIELDS, map(int, flags.split())))
    assert p.output_flags() == want
    f = _fields(p)
    p.write_output(tmp_path, 3, 0.0, f, hsml=p.hsml)
    head = (tmp_path / "nodes.csv.000003").read_text().split("\n")[0].rstrip()
    cols = ["x-coord", "", "y-coord"]
    for k, name in (("vx", "x-vel"), ("vy", "y-vel"), ("sxx", "sxx"), ("syy", "syy"),
                    ("sxy", "sxy"), ("szz", "szz"), ("strain", "strain"), ("disp", "disp"),
                    ("rho", "density"), ("sml", "sml")):
        if want[k]:
            cols.append(name)
    assert head.split(",") == cols
    row = (tmp_path / "nodes.csv.000003").read_text().split("\n")[1].rstrip().split(",")
    assert len(row) == len(cols) - 1
    if want["disp"]:
        d = f["displ"]
        assert row[cols.index("disp") - 1] == _f16_8(np.sqrt(d[0] ** 2 + d[1] ** 2))
