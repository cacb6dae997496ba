"""Reader for the reference's text field dumps (structure::Output_Scalar,
s_io_file.hpp:43-71), with the interface of the reference's own reader
(pyscript/read.py, class TextFile: get_config, get_data, get_coo_x,
get_coo_y, get_mat_val, get_arr_val), so fields written by the library
(carpio_gpu_output_scalar) and by the reference can be compared with the
same calls.

File layout: header lines "## Key : value" (Size, Dim, NX, NY), then one
line per normal cell, x fastest: "x, y, z, value".
"""
import re

import numpy as np

_HEADER = re.compile(r"##\s.+:.+")


class TextFile:
    def __init__(self, filename):
        with open(filename, "r") as f:
            self._lines = f.readlines()
        self._config = {}
        self._rows = []
        for line in self._lines:
            if _HEADER.match(line):
                # "## key : value" -> key, value (both stripped)
                key, val = line[3:-1].split(":")
                self._config[key.strip()] = val.strip()
            elif line.startswith("#"):
                continue
            else:
                row = []
                for tok in line.split(","):
                    tok = tok.strip()
                    try:
                        row.append(float(tok))
                    except ValueError:
                        pass
                if row:
                    self._rows.append(row)

    def get_config(self):
        return self._config

    def get_data(self):
        return self._rows

    def _n(self, key):
        return int(self._config[key])

    def get_coo_x(self):
        return [self._rows[i][0] for i in range(self._n("NX"))]

    def get_coo_y(self):
        if self._n("Dim") < 2:
            return [0]
        nx = self._n("NX")
        return [self._rows[j * nx][1] for j in range(self._n("NY"))]

    def get_mat_val(self):
        """values as rows of constant y: mat[j][i]"""
        assert self._n("Dim") == 2
        nx, ny = self._n("NX"), self._n("NY")
        return [[self._rows[j * nx + i][3] for i in range(nx)] for j in range(ny)]

    def get_arr_val(self):
        assert self._n("Dim") == 1
        return [self._rows[i][3] for i in range(self._n("NX"))]

    def field(self):
        """the values as an (nx, ny) array, x first like the library's fields"""
        return np.asarray(self.get_mat_val(), dtype=np.float64).T


def diff(file_a, file_b):
    """largest absolute difference of two dumps of the same grid (coordinates
    must agree as printed)"""
    a, b = TextFile(file_a), TextFile(file_b)
    ca, cb = a.get_config(), b.get_config()
    if (ca.get("NX"), ca.get("NY")) != (cb.get("NX"), cb.get("NY")):
        raise ValueError("dumps of different grids")
    ra, rb = np.asarray(a.get_data()), np.asarray(b.get_data())
    if not np.array_equal(ra[:, :3], rb[:, :3]):
        raise ValueError("cell coordinates differ")
    return float(np.max(np.abs(ra[:, 3] - rb[:, 3]))) if len(ra) else 0.0
