"""Device-side bounds checks of the element pass (debug flag EFE_DEVICE_CHECKS=1, read once per
process, so the checks run in a child process).  Indices read from the caller's arrays are checked
before use: a connectivity node outside [0, nNodes), a node DOF outside the DOF vector, a pair slot
+ block offset outside [0, nnz).  A bad index is skipped and reported (EFE_STATUS_BOUNDS, element
recorded); GPUAssembler raises IndexError.

The planted errors lie where even an unchecked access would stay inside the allocations (K and the
node-DOF map are padded), so the test cannot fault the GPU whatever the outcome; it asserts that the
checks caught them and skipped the writes.  With valid inputs and the checks on, the pass agrees
with the unchecked pass.
"""

import json
import os
import subprocess
import sys

import pytest

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, json, sys
import numpy as np, torch
sys.path.insert(0, ROOT)
from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes
from edelweissfe_gb300 import _lib as L

coords, conn, nodeDof, nDof = meshes.box(3, 3, 3, nNodes=8)
rng = np.random.default_rng(0)
dU = rng.uniform(-1, 1, nDof) * 1e-3
asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn)],
                   precision=PRECISION)
dev = asm.device
d = torch.tensor(dU, device=dev)
out = {}

def run(K, status):
    P, F = asm.constructDofVector(), asm.constructDofVector()
    L.check(asm.lib.efe_compute_elements(ctypes.byref(asm.mesh), asm._groups_c, 1, ctypes.c_void_p(d.data_ptr()),
            ctypes.c_void_p(d.data_ptr()), None, 0.0, asm.kPrecision, ctypes.c_void_p(K.data_ptr()),
            ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(status.data_ptr()), None),
            "efe_compute_elements")
    torch.cuda.synchronize()
    return P

# valid inputs, checks on
Pd, Kd, Fd = asm.constructDofVector(), asm.constructSystemMatrix(), asm.constructDofVector()
asm.computeElements(None, d, d, Pd, Kd, Fd)
out["valid_P"] = Pd.cpu().numpy().tolist()
out["valid_K_max"] = float(Kd.abs().max())
# a pair slot past nnz (K padded by 512 entries, so even an unchecked write would stay in the allocation)
slots = asm.groups[0]._dev["pairSlot"]
saved = slots.clone()
slots.view(len(conn), 8, 8)[5, 2, 3] = asm.nnz + 8
K = torch.zeros(asm.nnz + 512, dtype=asm.kdtype, device=dev)
st = torch.zeros(4, dtype=torch.int32, device=dev)
run(K, st)
s = st.cpu().numpy()
out["slot_status"] = [int(x) for x in s]
out["slot_pad_untouched"] = bool((K[asm.nnz:] == 0).all())
slots.copy_(saved)
# a connectivity node past nNodes (the node-DOF map padded with the valid DOF 0)
cn = asm.groups[0]._dev["conn"]
saved = cn.clone()
cn.view(len(conn), 8)[7, 4] = asm.nNodes + 3
pad = torch.cat([asm.nodeDof, torch.zeros(64, dtype=torch.int32, device=dev)])
asm.mesh.nodeDof = pad.data_ptr()
st.zero_()
run(torch.zeros(asm.nnz + 512, dtype=asm.kdtype, device=dev), st)
out["node_status"] = [int(x) for x in st.cpu().numpy()]
asm.mesh.nodeDof = asm.nodeDof.data_ptr()
cn.copy_(saved)
# the product API raises on the status bit
slots.view(len(conn), 8, 8)[5, 2, 3] = asm.nnz + 8
try:
    Kbig = torch.zeros(asm.nnz + 512, dtype=asm.kdtype, device=dev)  # a view of nnz entries with slack behind
    asm.launch(d, d, asm.constructDofVector(), Kbig[:asm.nnz], asm.constructDofVector())
    asm.check_status()
    out["raised"] = None
except IndexError as e:
    out["raised"] = str(e)
print("RESULT " + json.dumps(out))
"""


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bounds_checks_report_and_skip(precision):
    import numpy as np
    import torch

    from edelweissfe_gb300 import ElementGroup, GPUAssembler, meshes

    code = CHILD.replace("ROOT", repr(ROOT)).replace("PRECISION", repr(precision))
    env = dict(os.environ, EFE_DEVICE_CHECKS="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(next(l for l in r.stdout.splitlines() if l.startswith("RESULT "))[7:])
    # the planted slot: reported for element 5, the padding after nnz untouched
    assert out["slot_status"][0] & 16 and 0x7FFFFFFF - out["slot_status"][1] == 5
    assert out["slot_pad_untouched"]
    # the planted node: reported for element 7
    assert out["node_status"][0] & 16 and 0x7FFFFFFF - out["node_status"][1] == 7
    assert out["raised"] and "element 5" in out["raised"]
    # valid inputs with the checks on: the same pass as without them (this process: checks off)
    coords, conn, nodeDof, nDof = meshes.box(3, 3, 3, nNodes=8)
    dU = np.random.default_rng(0).uniform(-1, 1, nDof) * 1e-3
    asm = GPUAssembler(coords, nodeDof, nDof, [ElementGroup("C3D8", "vonmises", [210e3, 0.3, 250, 1000, 0, 0], conn)],
                       precision=precision)  # fmt: skip
    d = torch.tensor(dU, device=asm.device)
    P, K, F = asm.constructDofVector(), asm.constructSystemMatrix(), asm.constructDofVector()
    asm.computeElements(None, d, d, P, K, F)
    Pc = np.array(out["valid_P"])
    assert np.abs(Pc - P.cpu().numpy()).max() <= 1e-12 * np.abs(Pc).max()
