"""The reference's binary grid files (UNF): raw big-endian values, no header.

`.365.UNF0` climate files hold float32 values cell-major, [ncell][365]
(climateYearClass::read_climate_data_daily_per_year, source/climateYear.cpp:38-79;
VariableChannelGrid(cell, day) = data[cell * 365 + day], source/grid.h;
GridUNFAdapter, source/grid_io_adapters.h:42-129).  Used here to write such
files from synthetic forcing and to hand their raw bytes to
wg_upload_forcing_unf, which byte-swaps and transposes on the GPU.
"""
from __future__ import annotations

import numpy as np

# file names of the reference's daily climate input (climateYear.cpp:46-58)
CLIMATE_FILES = {"temp": "G_TEMP_H08_int_{year}.365.UNF0",
                 "prec": "G_GPCC_H08day_V20110128_{year}.365.UNF0",
                 "swrad": "G_SSRD_H08_int_{year}.365.UNF0"}


def write_unf0(path: str, cell_major: np.ndarray) -> None:
    """Write float values [ncell][nchannel] as a big-endian float32 UNF0 file."""
    np.ascontiguousarray(cell_major, dtype=">f4").tofile(path)


def read_unf0(path: str, ncell: int, nchannel: int) -> np.ndarray:
    """Read a UNF0 file as float32 [ncell][nchannel] (host byte order)."""
    a = np.fromfile(path, dtype=">f4", count=ncell * nchannel)
    if a.size != ncell * nchannel:
        raise ValueError(f"{path}: {a.size} values, expected {ncell * nchannel}")
    return a.reshape(ncell, nchannel).astype(np.float32)


def write_climate_year(directory: str, year: int, P, T, S) -> dict:
    """One year of day-major forcing [365][ncell] as the reference's three daily
    climate files; returns their paths by variable."""
    import os
    paths = {}
    for key, arr in (("prec", P), ("temp", T), ("swrad", S)):
        path = os.path.join(directory, CLIMATE_FILES[key].format(year=year))
        write_unf0(path, np.asarray(arr, np.float32).T)
        paths[key] = path
    return paths
