"""Reference file formats and inputs: Armadillo sparse binary (form_factors.bin),
sun-position text files, OBJ ingestion with the reference's normal
orientation and vertex scale."""
import numpy as np

from illum_gb300 import armaio, meshgen


def _csr(n, rng, density=0.05):
    rows, cols = np.nonzero(rng.random((n, n)) < density)
    vals = rng.random(rows.size)
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, rows + 1, 1)
    return np.cumsum(rowptr), cols.astype(np.int32), vals


def test_sparse_arma_round_trip_and_layout(tmp_path):
    rng = np.random.default_rng(5)
    rp, c, v = _csr(37, rng)
    p = tmp_path / "form_factors.bin"
    armaio.save_sparse(str(p), rp, c, v)
    raw = p.read_bytes()
    head, dims, body = raw.split(b"\n", 2)
    assert head == b"ARMA_SPM_BIN_FN008"
    n_rows, n_cols, nnz = (int(x) for x in dims.split())
    assert (n_rows, n_cols, nnz) == (37, 37, v.size)
    assert len(body) == 8 * nnz + 8 * nnz + 8 * (n_cols + 1)
    # compressed-column body: values, row indices, column pointers
    vals = np.frombuffer(body[:8 * nnz], np.float64)
    rows = np.frombuffer(body[8 * nnz:16 * nnz], np.uint64)
    colptr = np.frombuffer(body[16 * nnz:], np.uint64)
    dense = np.zeros((37, 37))
    for j in range(37):
        for k in range(colptr[j], colptr[j + 1]):
            dense[rows[k], j] = vals[k]
    ref = np.zeros((37, 37))
    for i in range(37):
        ref[i, c[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    assert np.array_equal(dense, ref)
    rp2, c2, v2, nc = armaio.load_sparse(str(p))
    assert nc == 37 and np.array_equal(rp2, rp) and np.array_equal(c2, c) and np.array_equal(v2, v)


def test_sparse_arma_empty(tmp_path):
    p = tmp_path / "e.bin"
    armaio.save_sparse(str(p), np.zeros(5, np.int64), np.zeros(0, np.int32), np.zeros(0))
    rp, c, v, nc = armaio.load_sparse(str(p))
    assert nc == 4 and rp.tolist() == [0, 0, 0, 0, 0] and c.size == 0 and v.size == 0


def test_sun_positions_file(tmp_path):
    p = tmp_path / "sun.txt"
    p.write_text("1.5e11 0 2e10 99\n-3e11 4e10 0 7\n")
    S = armaio.load_sun_positions(str(p), unit="m")
    assert S.shape == (2, 3)
    assert np.allclose(S, [[1.5e8, 0, 2e7], [-3e8, 4e7, 0]])
    assert np.array_equal(armaio.load_sun_positions(str(p)), np.array([[1.5e11, 0, 2e10], [-3e11, 4e10, 0]]))


def test_obj_normals_follow_vertex_normals_and_scale(tmp_path):
    # a quad (fan-split into two triangles) whose vertex normals point down
    # (-z): the cross-product normal (+z) is flipped, as obj_util.cpp:66-88
    p = tmp_path / "m.obj"
    p.write_text("o first\n"
                 "v 0 0 0\nv 100 0 0\nv 100 100 0\nv 0 100 0\n"
                 "vn 0 0 -1\nvn 0 0 -1\nvn 0 0 -1\nvn 0 0 -1\n"
                 "f 1//1 2//2 3//3 4//4\n"
                 "o second\n"
                 "v 0 0 5\nv 0 100 5\nv 100 0 5\n"
                 "vn 0 0 1\nvn 0 0 1\nvn 0 0 1\n"
                 "f 5 6 7\n")
    V, F, N = meshgen.load_obj(str(p))
    assert F.tolist() == [[0, 1, 2], [0, 2, 3]]
    assert np.allclose(V[1], [1.0, 0, 0])                      # vertices / 100
    assert np.allclose(N, [[0, 0, -1], [0, 0, -1]])
    V2, F2, N2 = meshgen.load_obj(str(p), shape_index=1, scale=1.0)
    assert F2.tolist() == [[4, 5, 6]]
    # (v1 - v0) x (v2 - v0) = (0,100,0) x (100,0,0) = -z; vertex normals +z: flipped
    assert np.allclose(N2, [[0, 0, 1]])


def test_cli_yaml_config_and_overrides(tmp_path):
    from illum_gb300 import cli
    y = tmp_path / "job.yaml"
    y.write_text("# thermal job\nnphi: 64\nthermal: true\nradiosity: yes\ndt: 120.5\n"
                 "depths: [0.01, 0.02, 0.05]\nrhoc:\n  - 1.0e6\nT0: init.bin\nsun_unit: km\n")
    cfg = cli.parse_yaml(y.read_text())
    assert cfg == {"nphi": 64, "thermal": True, "radiosity": True, "dt": 120.5, "depths": [0.01, 0.02, 0.05],
                   "rhoc": [1.0e6], "T0": "init.bin", "sun_unit": "km"}
    a = cli.resolve(["--config", str(y), "--nphi", "32", "--task", "horizons"])
    assert a.nphi == 32 and a.thermal is True and a.depths == [0.01, 0.02, 0.05] and a.rhoc == [1.0e6]
    assert a.T0 == "init.bin" and a.sun_unit == "km" and a.task == "horizons"
