"""Headless cluster debug views (vren_demo's show_clusters / show_clusters_geometry): the GPU views
against the CPU restatement bit for bit, and the host writers (PPM, PFM, OBJ, JSON, frame diff)."""
import json

import numpy as np
import pytest

import oracle
import vren_gb300.cluster_debug as cd


def oracle_frame(W=640, H=360, L=4096, seed=77):
    import vren_gb300.clustered_shading as cs
    import vren_gb300.scene as scene

    view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
    depth, normals = scene.depth_planes(seed, W, H)
    pos, li = scene.lights_near_camera(seed + 1, L)
    keys, refs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0)
    vp, bvh, lidx = oracle.cs_light_bvh(pos, li, L, view, 15)
    c, o, i, _ = oracle.cs_assign_lights(keys, W, H, view, bvh, L, lidx, vp)
    return view, {"keys": keys, "refs": refs, "counts": c, "offsets": o, "indices": i, "width": W, "height": H}


def test_decode_key():
    key = (5 << 26) | (17 << 16) | (3 << 8) | 9
    assert cd.decode_key(key) == {"ijk": [9, 3, 17], "normal": [0, 1, 2]}
    assert cd.decode_key(0x3F << 26)["normal"] is None


def test_writers_round_trip(tmp_path, native):
    rng = np.random.default_rng(1)
    img = rng.uniform(-0.2, 1.2, (5, 7, 4)).astype(np.float32)
    cd.write_ppm(tmp_path / "a.ppm", img)
    raw = (tmp_path / "a.ppm").read_bytes()
    assert raw.startswith(b"P6\n7 5\n255\n")
    px = np.frombuffer(raw[len(b"P6\n7 5\n255\n"):], np.uint8).reshape(5, 7, 3)
    assert np.array_equal(px, np.rint(np.clip(img[..., :3], 0, 1) * 255).astype(np.uint8))
    cd.write_pfm(tmp_path / "a.pfm", img)
    assert np.array_equal(cd.read_pfm(tmp_path / "a.pfm"), img[..., :3])
    _, fr = oracle_frame()
    verts = oracle.cs_show_clusters_geometry(oracle_frame()[0], fr["width"], fr["height"], fr["keys"][:3])
    cd.write_obj(tmp_path / "g.obj", verts)
    lines = (tmp_path / "g.obj").read_text().splitlines()
    assert sum(l.startswith("v ") for l in lines) == 96 and sum(l.startswith("l ") for l in lines) == 48
    cd.write_cluster_json(tmp_path / "c.json", fr)
    table = json.loads((tmp_path / "c.json").read_text())["clusters"]
    assert len(table) == len(fr["keys"])
    t = max(table, key=lambda r: r["light_count"])
    o, n = fr["offsets"][t["cluster"]], fr["counts"][t["cluster"]]
    assert t["lights"] == [int(x) for x in fr["indices"][o:o + n]]


def test_diff_frames_finds_planted_differences(tmp_path, native):
    """Mistakes planted in a copy of the oracle's outputs are found and located."""
    _, a = oracle_frame()
    b = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in a.items()}
    assert cd.diff_frames(a, b)["key_mismatch"] == 0
    c = int(np.argmax(a["counts"]))
    assert a["counts"][c] >= 2
    o = a["offsets"][c]
    b["indices"][o], b["indices"][o + 1] = a["indices"][o + 1], a["indices"][o]   # order swapped
    b["keys"][0] ^= 1                                                             # one key changed
    res = cd.diff_frames(a, b, out_dir=tmp_path)
    W = a["width"]
    assert res["key_mismatch"] == int((a["refs"] == 0).sum())
    assert res["light_mismatch"] == int((a["refs"] == c).sum()) - (int((a["refs"] == 0).sum()) if c == 0 else 0)
    assert (tmp_path / "mismatch.ppm").exists() and json.loads((tmp_path / "mismatch.json").read_text())
    bad = [r for r in res["clusters"] if "lights_a" in r]
    assert bad and bad[0]["lights_a"][:2] == [int(a["indices"][o]), int(a["indices"][o + 1])]
    p = bad[0]["pixel"]
    assert a["refs"][p[1] * W + p[0]] == c


def test_oracle_show_clusters_modes_are_functions_of_the_cluster(native):
    """Every mode's colour depends on the pixel's cluster alone (what the GPU's per-cluster table uses)."""
    _, fr = oracle_frame()
    for mode in range(7):
        img = oracle.cs_show_clusters(mode, fr["width"], fr["height"], fr["refs"], fr["keys"], fr["counts"],
                                      fr["offsets"], fr["indices"]).reshape(-1, 4)
        first = {}
        for p, r in enumerate(fr["refs"]):
            first.setdefault(int(r), p)
        rep = np.array([first[int(r)] for r in fr["refs"]])
        assert np.array_equal(img.view(np.uint32), img[rep].view(np.uint32))
