"""Oracle of the border-distance diagnostic (functions.py:58-97).

TEST INFRASTRUCTURE: only tests/ use this module. It restates
functions.distance_to_border with scipy's KD-tree: border vertices are the
ICON vertices with a -2 in cells_of_vertex (functions.py:88), both point sets
go to spherical ECEF with R = 6371.0087714 km (functions.py:89-97), and the
result is the chord distance to the nearest border vertex (functions.py:98-100).
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import cKDTree

RAD_E = 6371.0087714  # km, functions.py:89


def _ecef(lon, lat):
    return np.vstack((RAD_E * np.cos(lat) * np.cos(lon), RAD_E * np.cos(lat) * np.sin(lon),
                      RAD_E * np.sin(lat))).transpose()


def distance_to_border(clon, clat, vlon, vlat, cells_of_vertex):
    mask = np.any(np.asarray(cells_of_vertex) == -2, axis=0)
    if not mask.any():
        return np.full(np.asarray(clon).size, np.inf)
    tree = cKDTree(_ecef(np.asarray(vlon)[mask], np.asarray(vlat)[mask]))
    dist, _ = tree.query(_ecef(np.asarray(clon), np.asarray(clat)), k=1)
    return dist
