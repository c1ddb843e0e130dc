"""UNF climate files: the writer's byte order and layout, and the library's
reader (no GPU)."""
import os

import numpy as np


def test_unf0_round_trip_and_layout(tmp_path):
    from watergap2_gb300 import unf
    rng = np.random.default_rng(0)
    a = rng.normal(size=(7, 365)).astype(np.float32)          # [cell][day]
    path = os.path.join(tmp_path, "x.365.UNF0")
    unf.write_unf0(path, a)
    raw = open(path, "rb").read()
    assert len(raw) == 7 * 365 * 4
    # big-endian, cell-major: the first 4 bytes are cell 0 day 0
    assert raw[:4] == np.array([a[0, 0]], dtype=">f4").tobytes()
    assert raw[4:8] == np.array([a[0, 1]], dtype=">f4").tobytes()
    assert raw[:4] == np.array([a[0, 0]], dtype=np.float32).tobytes()[::-1]   # little-endian host
    assert np.array_equal(unf.read_unf0(path, 7, 365), a)


def test_library_reads_unf_files(tmp_path):
    from watergap2_gb300 import build, gpu, unf
    if not os.path.exists(gpu.LIB_PATH):
        build.build()
    P = np.arange(365 * 5, dtype=np.float32).reshape(365, 5)
    paths = unf.write_climate_year(str(tmp_path), 1990, P, P + 1, P + 2)
    assert os.path.basename(paths["prec"]) == "G_GPCC_H08day_V20110128_1990.365.UNF0"
    buf = gpu.read_unf(paths["temp"], 5 * 365 * 4)
    got = buf.view(">f4").reshape(5, 365)
    assert np.array_equal(got, (P + 1).T)
