import numpy as np

from ettk_gb300 import volume_list


def test_roundtrip(tmp_path):
    rows = [{"lwedge": -60.0, "uwedge": 60.0, "position": (32, 32, 32), "geometry": (64, 64, 64),
             "normal": (0, 0, 137.5), "matrix": np.eye(4), "magnification": (1, 1, 1), "cut_offset": 0,
             "filename": "particle_00001.mrc"},
            {"lwedge": -45.25, "uwedge": 70.0, "position": (10.5, 20, 30), "geometry": (32, 32, 32),
             "normal": (1, 2, 3), "matrix": np.arange(16).reshape(4, 4), "magnification": (1, 1, 1),
             "cut_offset": 2.5, "filename": "b.mrc"}]
    p = tmp_path / "vols.txt"
    volume_list.write(str(p), rows)
    txt = p.read_text().splitlines()
    assert txt[0].split("\t")[0] == "number" and len(txt[0].split("\t")) == 33
    assert len(txt[1].split("\t")) == 33
    back = volume_list.read(str(p))
    assert len(back) == 2
    assert back[1]["normal"] == (1.0, 2.0, 3.0) and back[1]["filename"] == "b.mrc"
    assert np.array_equal(back[1]["matrix"], np.arange(16).reshape(4, 4))
    assert back[0]["cut_offset"] == 0 and back[1]["cut_offset"] == 2.5
