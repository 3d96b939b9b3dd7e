"""The standalone Newton driver (solver.NISTGPU) on the CPU, against complete reference simulations.

The same Newton fixtures the GPU suite replays (tests/golden/newton: 17 of the reference's own test
inputs and two written for this purpose, recorded by running the reference), plus a run in which a
material point of the reference asks for a cutback (tests/golden/newton_cutback), with the oracle behind
GPUAssembler's interface (test infrastructure; the status word of a failed material point goes
through the product's own GPUAssembler.check_status) and SuperLU solves: the same increments,
Newton iterations per increment (cutbacks included) and converged displacements as the reference
(1e-9 of its largest displacement).  This puts the driver's increment, cutback and convergence
logic, its Dirichlet handling and its nodal and body loads under every CPU run; the GPU suite
replays the same fixtures with the CUDA element pass.
"""

import numpy as np
import pytest

import newton_cases as nc

torch = pytest.importorskip("torch")


class OracleDeviceAssembler:
    """The subset of GPUAssembler's interface the Newton driver uses, over the oracle, on CPU tensors."""

    def __init__(self, coords, nodeDof, nDof, groups):
        from oracle.assembly import Model

        self.device = torch.device("cpu")
        self.dim = np.asarray(coords).shape[1]
        self.nDof = int(nDof)
        self.groups = list(groups)
        recs, off = [], 0
        for g in self.groups:
            n = len(g.conn)
            recs.append(dict(elType=g.elType, kind=g.material, props=np.asarray(g.props, float), conn=g.conn,
                             thickness=np.broadcast_to(np.asarray(g.thickness, float), (n,)),
                             order=np.arange(off, off + n)))  # fmt: skip
            off += n
        self.model = Model(coords, nodeDof, nDof, recs)
        self.indptr_host, self.indices_host = self.model.indptr, self.model.indices
        self.nnz = len(self.indices_host)
        self.status = torch.zeros(4, dtype=torch.int32)
        self._ref = self.model.initial_state()
        self._temp = None

    def constructDofVector(self):
        return torch.zeros(self.nDof, dtype=torch.float64)

    def constructSystemMatrix(self):
        return torch.zeros(self.nnz, dtype=torch.float64)

    def launch(self, U_np, dU, P, K, F, time=None, dT=0.0):
        from edelweissfe_gb300 import _lib as L

        r = self.model.compute_elements(U_np.numpy(), dU.numpy(), self._ref)
        P += torch.from_numpy(r["P"])
        F += torch.from_numpy(r["F"])
        K += torch.from_numpy(r["Kdata"])
        self._temp = r["stateTemp"]
        if r["first_failed_element"] is not None:  # the device status word of a failed material point
            self.status[0] = int(self.status[0]) | L.EFE_STATUS_CUTBACK
            self.status[1] = max(int(self.status[1]), 0x7FFFFFFF - int(r["first_failed_element"]))
            self.status[2] = int(self.status[2]) + int(sum(np.count_nonzero(f) for f in r["fail"]))

    def check_status(self):
        from edelweissfe_gb300.assembly import GPUAssembler

        return GPUAssembler.check_status(self)

    def acceptLastState(self):
        from oracle.assembly import Model

        self._ref = Model.accept_state(self._temp)

    def computeBodyForce(self, P, force, elements=None):
        P += torch.from_numpy(self.model.body_force(np.asarray(force, float), elements))

    def assembleStiffnessCSR(self, K, host=True):
        import scipy.sparse as sp

        return sp.csr_matrix((K.numpy().copy(), self.indices_host.copy(), self.indptr_host.copy()),
                             shape=(self.nDof, self.nDof))  # fmt: skip


CASES = [(n, "newton") for n in nc.names()] + [(n, "newton_cutback") for n in nc.names("newton_cutback")]


@pytest.mark.parametrize("name,subdir", CASES)
def test_newton_driver_replays_the_reference_simulation(name, subdir):
    from edelweissfe_gb300.solver import NISTGPU

    case = nc.load(name, subdir)
    asm = OracleDeviceAssembler(case["coords"], case["node_dof"], int(case["nDof"]), nc.groups(case))
    stepper, dirichlets, nodeforces, bodyforces, ctl = nc.step_inputs(case)
    solver = NISTGPU(asm, linsolver="superlu", extrapolation=str(case["extrapolation"]), maxIter=ctl["maxIter"],
                     criticalIter=ctl["criticalIter"], maxGrowingIter=ctl["maxGrowingIter"])  # fmt: skip
    U = solver.solveStep(stepper, dirichlets, nodeforces, bodyforces, cutbackFactor=ctl["cutbackFactor"]).numpy()
    ours = [h["iterations"] if h["iterations"] is not None else -1 for h in solver.history]
    assert ours == [int(i[6]) for i in case["increments"]]
    progress = [h["timeStep"].stepProgress for h in solver.history]
    assert np.allclose(progress, case["increments"][:, 2], rtol=0, atol=1e-14)
    scale = np.abs(case["U_final"]).max()
    assert np.abs(U - case["U_final"]).max() <= 1e-9 * scale
    if "U_ref" in case:
        assert np.abs(U - case["U_ref"]).max() < 1e-6
