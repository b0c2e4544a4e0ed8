"""Loader of the known-answer cases extracted from the reference's unit tests."""
import json
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_cases.json")


def load(op=None):
    with open(PATH) as fh:
        cases = json.load(fh)["cases"]
    return [c for c in cases if op is None or c["op"] == op]


def case_id(c):
    return f"{c['name']}@{os.path.basename(c['file'])}:{c['line']}"


def f32(raster):
    return np.array([[np.nan if v is None else v for v in row] for row in raster], dtype=np.float32)


def u8(raster):
    return np.array(raster, dtype=np.uint8)


def arg(spec, dtype=np.float32):
    """A raster-or-scalar input of a case as a numpy array or a Python float."""
    if "raster" in spec:
        return np.array([[np.nan if v is None else v for v in row] for row in spec["raster"]], dtype=dtype)
    v = spec["scalar"]
    return np.dtype(dtype).type(float("nan") if v is None else v)
