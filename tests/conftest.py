import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    return sorted(os.path.basename(p)[:-5] for p in glob.glob(os.path.join(GOLDEN, "*.json")))


def load_golden(name):
    with open(os.path.join(GOLDEN, name + ".json")) as fh:
        d = json.load(fh)
    from mongeampere_gb300.mesh import GridMesh, TriMesh
    m = d["mesh"]
    if m["kind"] == "grid":
        mesh = GridMesh(np.array(m["gx"]), np.array(m["gy"]), np.array(m["values"]))
    else:
        mesh = TriMesh(m["vx"], m["vy"], m["values"], m["tri"])
    d["mesh_obj"] = mesh
    return d


def hessian_dict(rows, cols, vals):
    return {(int(i), int(j)): float(v) for i, j, v in zip(rows, cols, vals)}


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O
