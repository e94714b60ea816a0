"""VTK image output, the interface of utils/dump_vtk.py:1-64 of the reference.

The reference builds a vtkImageData of dimensions (grid_size_z, grid_size_r, 1)
and writes it with vtkXMLImageDataWriter, the fields as the components of one
point-data array named "softy" (component i named field_names_list[i], field
i flattened in C order, so z varies fastest). The `vtk` package is not a
dependency here: this module writes the same VTK XML ImageData file (.vti)
itself, FP64, little-endian, base64 inline binary with a UInt64 byte-count
header, so ParaView and VTK readers open it as they open the reference's
files. Fields may be numpy arrays or torch tensors (device tensors are
copied to the host).
"""
import base64
from dataclasses import dataclass, field

import numpy as np


@dataclass
class _ImageData:
    dims: tuple
    origin: tuple = (0.0, 0.0, 0.0)
    spacing: tuple = (1.0, 1.0, 1.0)


@dataclass
class _PointArray:
    name: str = "softy"
    component_names: list = field(default_factory=list)


class _XMLImageDataWriter:
    """Writes one _ImageData with one point array per call."""

    def write(self, filename, image, array, data):
        nx, ny, nz = image.dims
        extent = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
        raw = np.ascontiguousarray(data, dtype="<f8").tobytes()
        payload = base64.b64encode(np.uint64(len(raw)).astype("<u8").tobytes() + raw)
        names = " ".join(f'ComponentName{i}="{n}"' for i, n in enumerate(array.component_names))
        head = (
            '<?xml version="1.0"?>\n'
            '<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" '
            'header_type="UInt64">\n'
            f'  <ImageData WholeExtent="{extent}" '
            f'Origin="{" ".join(repr(float(v)) for v in image.origin)}" '
            f'Spacing="{" ".join(repr(float(v)) for v in image.spacing)}">\n'
            f'    <Piece Extent="{extent}">\n'
            f'      <PointData>\n'
            f'        <DataArray type="Float64" Name="{array.name}" '
            f'NumberOfComponents="{data.shape[1]}" {names} format="binary">\n'
        )
        tail = ("\n        </DataArray>\n      </PointData>\n      <CellData>\n"
                "      </CellData>\n    </Piece>\n  </ImageData>\n</VTKFile>\n")
        with open(filename, "wb") as f:
            f.write(head.encode())
            f.write(payload)
            f.write(tail.encode())


def vtk_init(grid_size_z, grid_size_r):
    """Initialises the writer (dump_vtk.py:5-29): image data of dimensions
    (grid_size_z, grid_size_r, 1), the point array, the writer."""
    return _ImageData((int(grid_size_z), int(grid_size_r), 1)), _PointArray(), \
        _XMLImageDataWriter()


def _host(a):
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64)


def vtk_write(filename, vtk_image_data, temp_vtk_array, writer, field_names_list, field_list,
              grid_size_z, grid_size_r):
    """Writes `field_list` as the components of the point array "softy"
    (dump_vtk.py:32-64)."""
    n = int(grid_size_z) * int(grid_size_r)
    if len(field_names_list) != len(field_list):
        raise ValueError("one name per field")
    cols = []
    for name, f in zip(field_names_list, field_list):
        a = _host(f).reshape(-1)
        if a.size != n:
            raise ValueError(f"field {name!r} has {a.size} values, the image {n}")
        cols.append(a)
    temp_vtk_array.name = "softy"
    temp_vtk_array.component_names = list(field_names_list)
    data = np.stack(cols, axis=1) if cols else np.zeros((n, 0))
    writer.write(filename, vtk_image_data, temp_vtk_array, data)


def read_vti(filename):
    """Reads a file written by vtk_write back: {component name: (ny, nx)
    array} plus "_dims". For tests and post-processing without VTK."""
    import xml.etree.ElementTree as ET
    root = ET.parse(filename).getroot()
    img = root.find("ImageData")
    ext = [int(v) for v in img.get("WholeExtent").split()]
    nx, ny = ext[1] - ext[0] + 1, ext[3] - ext[2] + 1
    arr = img.find("Piece/PointData/DataArray")
    nc = int(arr.get("NumberOfComponents"))
    raw = base64.b64decode(arr.text.strip())
    nbytes = int(np.frombuffer(raw[:8], dtype="<u8")[0])
    data = np.frombuffer(raw[8:8 + nbytes], dtype="<f8").reshape(-1, nc)
    out = {"_dims": (nx, ny), "_name": arr.get("Name")}
    for i in range(nc):
        out[arr.get(f"ComponentName{i}")] = data[:, i].reshape(ny, nx)
    return out
