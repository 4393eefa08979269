"""Headless export of the particle state, in the reference's output formats.

``export_csv`` writes the columns and header of the reference's CSV export
(eng/ui_sim.py:293-298) and ``export_vtk`` a VTK XML unstructured grid of vertex cells
with every array of ``ParticleSystem.dump()`` as point data - the file the reference
writes through pyevtk's ``pointsToVTK`` (eng/ui_sim.py:300-304).  File names follow the
reference's ``sim.csv.<stamp>.csv`` / ``sim.vtk.<stamp>.vtu`` pattern inside ``simpath``.
Both read the device state through ``dump()`` (field views copied to the host).
"""
import os

import numpy as np

CSV_COLUMNS = ("id0", "objId", "material", "pos.x", "pos.y", "pos.z", "vel.x", "vel.y", "vel.z", "density",
               "stress.xx", "stress.yy", "stress.zz", "stress.xy", "stress.yz", "stress.zx", "strain_equ")


def export_csv(stamp, simpath, case):
    """sim.csv.<stamp>.csv with the reference's 17 columns (ids, position, velocity,
    density, stress components, equivalent strain)."""
    pos, data = case.ps.dump()
    merged = {**data, **pos}
    table = np.array([merged[c] for c in CSV_COLUMNS], dtype=np.float64).T
    path = os.path.join(simpath, f"sim.csv.{stamp}.csv")
    np.savetxt(path, table, delimiter=",", header=", ".join(CSV_COLUMNS))
    return path


def _vtk_type(a):
    if a.dtype == np.float64:
        return "Float64"
    if a.dtype == np.float32:
        return "Float32"
    if a.dtype == np.int64:
        return "Int64"
    return "Int32"


def export_vtk(stamp, simpath, case):
    """sim.vtk.<stamp>.vtu: points, one vertex cell per particle, every dump() array as
    point data (raw appended little-endian binary with 64-bit block headers)."""
    pos, data = case.ps.dump()
    n = pos["pos.x"].shape[0]
    pts = np.stack([pos["pos.x"], pos["pos.y"], pos["pos.z"]], axis=1).astype(np.float64)
    cells = [("connectivity", np.arange(n, dtype=np.int64)), ("offsets", np.arange(1, n + 1, dtype=np.int64)),
             ("types", np.ones(n, dtype=np.uint8))]
    point_data = [(k, np.ascontiguousarray(v)) for k, v in data.items()]
    offset = 0
    pieces = []

    def add(arr):
        nonlocal offset
        raw = np.ascontiguousarray(arr).tobytes()
        pieces.append(np.uint64(len(raw)).tobytes() + raw)
        start = offset
        offset += 8 + len(raw)
        return start

    xml = ['<?xml version="1.0"?>',
           '<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
           '<UnstructuredGrid>', f'<Piece NumberOfPoints="{n}" NumberOfCells="{n}">', "<Points>"]
    xml.append(f'<DataArray type="Float64" NumberOfComponents="3" format="appended" offset="{add(pts)}"/>')
    xml += ["</Points>", "<Cells>"]
    for name, arr in cells:
        t = "UInt8" if arr.dtype == np.uint8 else "Int64"
        xml.append(f'<DataArray type="{t}" Name="{name}" format="appended" offset="{add(arr)}"/>')
    xml += ["</Cells>", "<PointData>"]
    for name, arr in point_data:
        xml.append(f'<DataArray type="{_vtk_type(arr)}" Name="{name}" format="appended" offset="{add(arr)}"/>')
    xml += ["</PointData>", "</Piece>", "</UnstructuredGrid>", '<AppendedData encoding="raw">']
    path = os.path.join(simpath, f"sim.vtk.{stamp}.vtu")
    with open(path, "wb") as f:
        f.write(("\n".join(xml) + "\n_").encode())
        for p in pieces:
            f.write(p)
        f.write(b"\n</AppendedData>\n</VTKFile>\n")
    return path
