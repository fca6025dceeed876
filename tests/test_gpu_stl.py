"""The STL reader (records decoded and vertices merged on the GPU) against the
reference's read_stl (fixtures made by it) and the oracle restatement: points bit for
bit in first-occurrence order, triangles, error messages; in memory and through
read_plc; and a read mesh voxelizing like the same arrays given directly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _arrays(plc):
    return plc.points, plc.triangles


def test_fixtures_in_memory_and_files(cm, golden, tmp_path):
    g = golden("stl")
    for name in g["names"]:
        name = str(name)
        data = g[name + "_bytes"].tobytes()
        want_err = str(g[name + "_error"])
        for how in ("memory", "file"):
            if how == "memory":
                call = lambda: cm.plc_from_stl(data)
            else:
                path = tmp_path / (name + ".stl")
                path.write_bytes(data)
                call = lambda: cm.read_plc(str(path))
            if want_err:
                with pytest.raises(RuntimeError) as e:
                    call()
                assert str(e.value) == want_err, (name, how)
                continue
            pts, tri = _arrays(call())
            assert np.array_equal(pts.view(np.uint64), g[name + "_points"].view(np.uint64)), (name, how)
            assert np.array_equal(tri, g[name + "_triangles"]), (name, how)


@pytest.mark.parametrize("fmt", ["binary", "ascii"])
def test_large_meshes_match_oracle(cm, orc, fmt):
    from cybermeshgenerator_gb300 import workloads as W
    if fmt == "binary":
        p, t = W.ellipsoid_field(n=160, seed=8)          # 204,800 triangles
        data = W.stl_binary(p, t)
    else:
        p, t = W.sh_sphere()                              # 65,024 triangles, ~10 MB of text
        data = W.stl_ascii(p, t, fmt="{:.17g}", comments=True)
    want_p, want_t, err = orc.stl_read(data)
    assert err == ""
    got_p, got_t = _arrays(cm.plc_from_stl(data))
    assert np.array_equal(got_p.view(np.uint64), want_p.view(np.uint64))
    assert np.array_equal(got_t, want_t)
    # every STL vertex is merged: a closed mesh of V points reads back as V points
    assert len(got_p) == len(np.unique(p.astype(np.float32 if fmt == "binary" else np.float64), axis=0))


def test_read_mesh_voxelizes_like_its_arrays(cm):
    from cybermeshgenerator_gb300 import workloads as W
    p, t = W.jittered_icosphere(3, 0.02, seed=1)
    plc = cm.plc_from_stl(W.stl_binary(p, t))
    q, u = _arrays(plc)
    a = cm.voxelize_ex(plc, resolution=48, pad=2, outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32)
    b = cm.voxelize_ex(cm.PLC.from_arrays(q, u), resolution=48, pad=2,
                       outputs=cm.OUT_OCCUPANCY | cm.OUT_SDF_F32)
    assert np.array_equal(a.occupancy, b.occupancy)
    assert np.array_equal(a.sdf32, b.sdf32)
    assert a.occupancy.sum() > 0
