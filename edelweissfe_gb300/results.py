"""Field output from the device state: one result of many elements and quadrature points in one gather.

`ElementResultCollector` mirrors the reference's collector (`edelweissfe/utils/elementresultcollector.pyx`):
constructed once for a list of elements, a range of quadrature points and a result name, it returns
on every `getCurrentResults()` the array ``[elements, quadraturePoints, resultSize]`` (``[elements,
resultSize]`` for a single quadrature point).  The reference fills that table by walking one
persistent numpy view per (element, point); here the state already lives structure-of-arrays on the
GPU, so the table is one indexed gather of the accepted state (the reference's views point into
``_stateVarsRef``, `displacementelement/element.py:222-235, 386-409`) followed by one device-to-host
copy.  Result names: "stress" and "strain" (state fields 0-5 and 6-11), and the material's own
result in field 12: "kappa" (von Mises, `vonmises.py:281-298`) or "energy" (Neo-Hooke,
`neohookepencegouformulationa.py:168-185`).
"""

import numpy as np
import torch

_FIELDS = {"stress": (0, 6), "strain": (6, 12), "kappa": (12, 13), "energy": (12, 13)}


class ElementResultCollector:
    """elements: global element indices (the assembler's element order); quadraturePoints: range or
    list of point numbers; result: "stress", "strain", "kappa" or "energy"."""

    def __init__(self, assembler, elements, quadraturePoints, result, accepted=True):
        if result not in _FIELDS:
            raise KeyError(f"unknown result {result!r}")
        self.asm = assembler
        self.result = result
        self.accepted = accepted
        self.nEls = len(elements)
        qps = np.asarray(list(quadraturePoints), np.int64)
        self.nGauss = len(qps)
        f0, f1 = _FIELDS[result]
        self.nSize = f1 - f0
        elements = np.asarray(elements, np.int64)
        dev = assembler.device
        self._parts = []  # (group, field slice, columns [k], output rows [k])
        for g in assembler.groups:
            d = g._dev
            off, n = d["offset"], len(g.conn)
            sel = np.nonzero((elements >= off) & (elements < off + n))[0]
            if len(sel) == 0:
                continue
            nInt = d["type"].nInt
            if qps.max(initial=-1) >= nInt or qps.min(initial=0) < 0:
                raise IndexError("quadrature point out of range")
            if f1 > d["stateRef"].shape[0]:
                raise KeyError(f"{result!r} does not exist for the material of group {g.name or g.elType}")
            cols = ((elements[sel] - off)[:, None] * nInt + qps[None, :]).ravel()
            rows = (sel[:, None] * self.nGauss + np.arange(self.nGauss)[None, :]).ravel()
            self._parts.append((g, slice(f0, f1), torch.from_numpy(cols).to(dev), torch.from_numpy(rows).to(dev)))
        covered = sum(len(p[3]) for p in self._parts)
        if covered != self.nEls * self.nGauss:
            raise IndexError("an element index is outside the assembler's elements")
        self._table = torch.empty((self.nEls * self.nGauss, self.nSize), dtype=torch.float64, device=dev)

    def getCurrentResults(self, device=False):
        """The current table: a host numpy array (device=False) or the device tensor (device=True)."""
        for g, fs, cols, rows in self._parts:
            s = g._dev["stateRef" if self.accepted else "stateTemp"]
            self._table[rows] = s[fs][:, cols].T
        t = self._table.view(self.nEls, self.nGauss, self.nSize)
        if self.nGauss == 1:
            t = t.view(self.nEls, self.nSize)
        return t if device else t.cpu().numpy()
