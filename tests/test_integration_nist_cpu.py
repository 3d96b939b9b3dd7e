"""The NIST subclass of the integration layer (make_nist_gpu) inside complete reference simulations,
on the CPU.

The reference's finiteElementSimulation runs an input file with ``*solver, solver=NISTGPU``, the
subclass registered as a maintainer would (a solver module plus a solverLibrary entry; both in
memory here, nothing is written to the reference tree), with the oracle behind GPUAssembler's
interface as its assembler (test infrastructure: this exercises the subclass's control flow --
array extraction, element pass hand-off, CSR hand-off, acceptance, state write-back and, in the
second step of the von Mises case, read-back, cutback translation -- not the CUDA kernels, which the GPU tests cover).  The run must reproduce the
reference's own NIST run of the same input: final displacements, every increment's Newton
iterations, and the field outputs that read the written-back state -- on inputs written here and
on all 17 edelweiss-provider test inputs of the reference (`testfiles/`).
Needs the reference source tree, named by the EDELWEISSFE_ROOT environment variable; skipped when
it is unset.
"""

import os
import sys
import types
from types import SimpleNamespace

import numpy as np
import pytest

REF = os.environ.get("EDELWEISSFE_ROOT", "")
pytestmark = [
    pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "edelweissfe")),
                       reason="EDELWEISSFE_ROOT (the reference source tree) is not set"),  # fmt: skip
    pytest.mark.filterwarnings("ignore::PendingDeprecationWarning"),  # numpy.matrix inside the reference
]
torch = pytest.importorskip("torch")

J2_CUBE = """
*material, name=vonmises, id=vonmises, provider=edelweiss
210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0
*job, name=j2job, domain=3d
*solver, solver={solver}, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX=3
nY=3
nZ=2
lX=1
lY=1
lZ=1
elProvider=edelweiss
elType=C3D8
*section, name=section1, material=vonmises, type=solid
all
*fieldOutput
create=perElement, name=stress, elSet=gen_all, result=stress, quadraturePoint=0:8
*step, solver=theSolver, maxInc=0.25, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=linear, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 2=0.0
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0
dirichlet, name=back, nSet=gen_back, field=displacement, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=0.006
*step, solver=theSolver, maxInc=0.5, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=linear, linsolver=superlu
dirichlet, name=top, nSet=gen_top, field=displacement, 2=0.009
"""

J2_CUTBACK = """
*material, name=vonmises, id=vonmises, provider=edelweiss
210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0
*job, name=j2job, domain=3d
*solver, solver={solver}, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX=2
nY=2
nZ=2
lX=1
lY=1
lZ=1
elProvider=edelweiss
elType=C3D8
*section, name=section1, material=vonmises, type=solid
all
*fieldOutput
create=perElement, name=stress, elSet=gen_all, result=stress, quadraturePoint=0:8
*step, solver=theSolver, maxInc=1.0, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=linear, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 2=0.0
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0
dirichlet, name=back, nSet=gen_back, field=displacement, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=0.1
"""

TWO_SECTIONS = """
*material, name=vonmises, id=vonmises, provider=edelweiss
210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0
*material, name=linearelastic, id=soft, provider=edelweiss
70000.0, 0.25
*job, name=j2job, domain=3d
*solver, solver={solver}, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX=3
nY=2
nZ=2
lX=1
lY=1
lZ=1
elProvider=edelweiss
elType=C3D8
*section, name=section1, material=vonmises, type=solid
gen_bottom
*section, name=section2, material=soft, type=solid
gen_top
*fieldOutput
create=perElement, name=stress, elSet=gen_all, result=stress, quadraturePoint=0:8
*step, solver=theSolver, maxInc=0.25, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=linear, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 2=0.0
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0
dirichlet, name=back, nSet=gen_back, field=displacement, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=0.006
"""

NH_BLOCK = """
*material, name=neohookewa, id=nh, provider=edelweiss
384.6153846, 833.3333333
*job, name=nhjob, domain=3d
*solver, solver={solver}, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX=2
nY=3
nZ=2
lX=1
lY=1
lZ=1
elProvider=edelweiss
elType=C3D8TL
*section, name=section1, material=nh, type=solid
all
*fieldOutput
create=perElement, name=stress, elSet=gen_all, result=stress, quadraturePoint=0:8
*step, solver=theSolver, maxInc=0.34, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=off, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 1=0.0, 2=0.0, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=-0.08
"""


class OracleAssembler:
    """GPUAssembler's interface over the oracle: device-layout state tensors ([field][element * nInt
    + qp]) in `groups[i]._dev`, torch DOF vectors and CSR data, the reference's CSR pattern."""

    def __init__(self, coords, nodeDof, nDof, groups, precision="fp64"):
        from oracle.assembly import Model
        from oracle import library

        self.nDof = int(nDof)
        self.nodeDof_host = np.asarray(nodeDof)
        recs, off = [], 0
        self.groups = []
        for g in groups:
            n = len(g.conn)
            recs.append(dict(elType=g.elType, kind=g.material, props=g.props, conn=g.conn, thickness=g.thickness,
                             order=np.arange(off, off + n)))  # fmt: skip
            nInt = library.get(g.elType)["nInt"]
            self.groups.append(SimpleNamespace(elType=g.elType, material=g.material, props=g.props, conn=g.conn,
                                               thickness=g.thickness,
                                               _dev={"offset": off, "type": SimpleNamespace(nInt=nInt)}))  # fmt: skip
            off += n
        self.model = Model(coords, nodeDof, nDof, recs)
        init = self.model.initial_state()
        self._eold = [st.get("Eold") for st in init]
        self._enew = list(self._eold)
        for g, st in zip(self.groups, init):
            E, nInt, S = st["state"].shape
            g._dev["stateRef"] = torch.zeros((S, E * nInt), dtype=torch.float64)
            g._dev["stateTemp"] = torch.zeros((S, E * nInt), dtype=torch.float64)

    def constructDofVector(self):
        return torch.zeros(self.nDof, dtype=torch.float64)

    def constructSystemMatrix(self):
        return torch.zeros(len(self.model.indices), dtype=torch.float64)

    def group_state(self, i, which="temp"):
        from edelweissfe_gb300.assembly import GPUAssembler

        return GPUAssembler.group_state(self, i, which)

    def computeElements(self, elements, U_np, dU, P, K, F, timeStep=None):
        from edelweissfe_gb300.exceptions import CutbackRequest
        from oracle.exceptions import CutbackRequest as OracleCutback

        ref = []
        for i, g in enumerate(self.groups):
            d = dict(state=self.group_state(i, "ref").copy())
            if self._eold[i] is not None:
                d["Eold"] = self._eold[i]
            ref.append(d)
        try:
            r = self.model.compute_elements_or_raise(U_np.numpy(), dU.numpy(), ref)
        except OracleCutback as e:  # what the device status word turns into on the GPU path
            raise CutbackRequest(str(e), e.cutbackSize) from e
        P += torch.from_numpy(r["P"])
        F += torch.from_numpy(r["F"])
        K += torch.from_numpy(r["Kdata"])
        for i, (g, st) in enumerate(zip(self.groups, r["stateTemp"])):
            E, nInt, S = st["state"].shape
            g._dev["stateTemp"].copy_(torch.from_numpy(st["state"].reshape(E * nInt, S).T.copy()))
            self._enew[i] = st.get("Enew")
        return P, K, F

    def assembleStiffnessCSR(self, K, host=True):
        import scipy.sparse as sp

        return sp.csr_matrix((K.numpy().copy(), self.model.indices.copy(), self.model.indptr.copy()),
                             shape=(self.nDof, self.nDof))  # fmt: skip

    def acceptLastState(self):
        for i, g in enumerate(self.groups):
            g._dev["stateRef"].copy_(g._dev["stateTemp"])
            if self._enew[i] is not None:
                self._eold[i] = self._enew[i]


@pytest.fixture(scope="module")
def ref():
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden

    make_golden.setup_reference(REF)
    return make_golden


def _simulate(inp, tmp_path):
    import edelweissfe.solvers.nonlinearimplicitstatic as nis
    from edelweissfe.drivers.inputfiledrivensimulation import finiteElementSimulation
    from edelweissfe.utils.inputfileparser import parseInputFile

    its = []
    orig = nis.NIST.solveIncrement

    def counted(self, *a, **k):  # Newton iterations of accepted increments, exception names of the others
        try:
            out = orig(self, *a, **k)
        except Exception as e:
            its.append(type(e).__name__)
            raise
        its.append(out[3])
        return out

    nis.NIST.solveIncrement = counted
    path = os.path.join(tmp_path, "job.inp")
    with open(path, "w") as f:
        f.write(inp)
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        model, foc = finiteElementSimulation(parseInputFile(path), verbose=False, suppressPlots=True)
    finally:
        os.chdir(cwd)
        nis.NIST.solveIncrement = orig
    U = np.hstack([f["U"].flatten() for f in model.nodeFields.values()])
    return U, its, np.asarray(foc.fieldOutputs["stress"].getResultHistory())


@pytest.mark.parametrize("inp", [J2_CUBE, J2_CUTBACK, TWO_SECTIONS, NH_BLOCK],
                         ids=["c3d8-vonmises", "c3d8-vonmises-cutback", "two-sections", "c3d8tl-neohooke"])  # fmt: skip
def test_subclass_reproduces_the_reference_simulation(ref, inp, tmp_path):
    import edelweissfe.config.solvers as solvers
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    from edelweissfe_gb300.integration import make_nist_gpu

    U0, its0, S0 = _simulate(inp.format(solver="NIST"), tmp_path)
    module = types.ModuleType("edelweissfe.solvers.nonlinearimplicitstaticgpu")
    module.NISTGPU = make_nist_gpu(NIST, precision="fp64", assemblerClass=OracleAssembler)
    sys.modules[module.__name__] = module
    solvers.solverLibrary["NISTGPU"] = "nonlinearimplicitstaticgpu"
    try:
        U1, its1, S1 = _simulate(inp.format(solver="NISTGPU"), tmp_path)
    finally:
        solvers.solverLibrary.pop("NISTGPU", None)
        sys.modules.pop(module.__name__, None)
    assert its1 == its0 and len(its0) >= 3
    if inp is J2_CUTBACK:  # a material point's cutback request, handled by the reference's solveStep
        assert "CutbackRequest" in its0
    assert np.abs(U1 - U0).max() <= 1e-10 * np.abs(U0).max()
    assert S1.shape == S0.shape and np.abs(S0).max() > 0
    assert np.abs(S1 - S0).max() <= 1e-9 * np.abs(S0).max()  # field output through the written-back state


def test_cutback_reaches_the_reference_as_its_own_exception(ref):
    """A material point's cutback on the GPU path (this package's CutbackRequest) is raised into the
    reference's solveStep as the CutbackRequest class NIST's module catches."""
    import edelweissfe.utils.exceptions as refexc
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    from edelweissfe_gb300.exceptions import CutbackRequest
    from edelweissfe_gb300.integration import make_nist_gpu

    class Failing:
        def __init__(self, *a, **k):
            pass

        def constructDofVector(self):
            return torch.zeros(3, dtype=torch.float64)

        def constructSystemMatrix(self):
            return torch.zeros(1, dtype=torch.float64)

        def computeElements(self, *a, **k):
            raise CutbackRequest("material point failed in element 0", 0.5)

    cls = make_nist_gpu(NIST, assemblerClass=Failing)
    solver = cls.__new__(cls)
    solver._gpuAssembler, solver.theDofManager = Failing(), None
    solver._gpuDofManager, solver._gpuElements = None, []
    with pytest.raises(refexc.CutbackRequest) as e:
        solver.computeElements({}, np.zeros(3), np.zeros(3), np.zeros(3), None, np.zeros(3), None)
    assert e.value.cutbackSize == 0.5 and "element 0" in str(e.value)


def test_models_with_constraints_are_refused(ref):
    """assembleConstraints adds to the host VIJ matrix, which the subclass does not assemble: a model
    with constraints is refused before the step runs instead of solving with a tangent that lacks them."""
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    from edelweissfe_gb300.integration import make_nist_gpu

    cls = make_nist_gpu(NIST)
    solver = cls.__new__(cls)
    model = SimpleNamespace(constraints={"tie": object()}, advanceToTime=lambda t: None)
    with pytest.raises(NotImplementedError, match="constraints"):
        solver.solveStep(None, model, None, [])


def test_assembler_is_kept_across_steps_and_rebuilt_with_the_state_on_changes(ref):
    """NIST builds a new DofManager every step: the same numbering keeps the assembler (and its device
    state); a changed model (here a material property) builds a new one that starts from the state
    the element objects hold."""
    from edelweissfe.numerics.dofmanager import DofManager
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    from test_integration_cpu import _prepared

    from edelweissfe_gb300.integration import make_nist_gpu

    model, dm = _prepared(ref, 3, "boxGen", ["nX=2", "nY=1", "nZ=1"], "C3D8", "vonmises",
                          [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0], 0.0, [0.5, 1.0, 1.0], 1, [0] * 3, [1] * 3)  # fmt: skip

    def new_dof_manager():
        return DofManager(model.nodeFields.values(), [], model.elements.values(), [], model.nodeSets.values())

    cls = make_nist_gpu(NIST, assemblerClass=OracleAssembler)
    solver = cls.__new__(cls)
    solver.theDofManager = dm
    first = solver._gpu(model.elements)
    solver.theDofManager = new_dof_manager()
    assert solver._gpu(model.elements) is first
    elements = list(model.elements.values())
    for k, el in enumerate(elements):
        el._stateVarsRef[:, 0] = 3.0 + k
    elements[0].material._E = 200000.0  # the section's shared material object
    solver.theDofManager = new_dof_manager()
    second = solver._gpu(model.elements)
    assert second is not first and second.groups[0].props[0][0] == 200000.0
    assert np.array_equal(second.group_state(0, "ref"), np.stack([el._stateVarsRef for el in elements]))


REFERENCE_CASES = [
    "CantileverBeamQuad4", "CantileverBeamQuad8", "CantileverBeamHexa8", "CantileverBeamVonMisesPE",
    "CantileverBeamQuad8NeoHookeWa", "CantileverBeamQuad8NeoHookeWb", "CantileverBeamQuad8NeoHookeWc",
    "FixedDisplacementQuad4", "FixedDisplacementQuad8", "SimpleBeamHexa8", "SimpleBeamQuad4", "SimpleBeamQuad8",
    "TensionBarHexa8", "TensionBarQuad4", "TensionBarQuad8", "WallShearHexa8", "WallShearHexa20",
]  # fmt: skip


@pytest.fixture(scope="module")
def superlu_for_pardiso():
    """The reference's default linear solver is PARDISO (not installed): SciPy's SuperLU in its place,
    in memory, for both runs of a comparison."""
    import scipy.sparse.linalg as sla

    name = "edelweissfe.linsolve.pardiso.pardiso"
    saved = sys.modules.get(name)
    stub = types.ModuleType(name)
    stub.pardisoSolve = lambda A, b: sla.spsolve(A, b, use_umfpack=False)
    sys.modules[name] = stub
    yield
    if saved is None:
        sys.modules.pop(name, None)
    else:
        sys.modules[name] = saved


def _run_case(case, solver, tmp_path):
    import shutil

    import edelweissfe.solvers.nonlinearimplicitstatic as nis
    from edelweissfe.drivers.inputfiledrivensimulation import finiteElementSimulation
    from edelweissfe.utils.inputfileparser import parseInputFile

    wd = os.path.join(tmp_path, f"{case}_{solver}")
    shutil.copytree(os.path.join(REF, "testfiles", case), wd)
    path = os.path.join(wd, "test.inp")
    with open(path) as f:
        text = f.read()
    with open(path, "w") as f:
        f.write(text.replace("solver=NIST,", f"solver={solver},"))
    its = []
    orig = nis.NIST.solveIncrement

    def counted(self, *a, **k):
        out = orig(self, *a, **k)
        its.append(out[3])
        return out

    nis.NIST.solveIncrement = counted
    cwd = os.getcwd()
    os.chdir(wd)
    try:
        model, foc = finiteElementSimulation(parseInputFile(path), verbose=False, suppressPlots=True)
    finally:
        os.chdir(cwd)
        nis.NIST.solveIncrement = orig
    U = np.hstack([f["U"].flatten() for f in model.nodeFields.values()])
    results = {name: np.asarray(fo.getLastResult(), float) for name, fo in foc.fieldOutputs.items()}
    return U, its, results


@pytest.mark.parametrize("case", REFERENCE_CASES)
def test_subclass_runs_the_reference_test_inputs(ref, superlu_for_pardiso, case, tmp_path):
    """The reference's own edelweiss-provider test inputs (testfiles/<case>/test.inp) with the
    solver switched to the GPU subclass: same displacements, Newton iterations and field outputs
    (per-element and per-node, through the written-back state) as with NIST."""
    import edelweissfe.config.solvers as solvers
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST

    from edelweissfe_gb300.integration import make_nist_gpu

    U0, its0, R0 = _run_case(case, "NIST", tmp_path)
    module = types.ModuleType("edelweissfe.solvers.nonlinearimplicitstaticgpu")
    module.NISTGPU = make_nist_gpu(NIST, precision="fp64", assemblerClass=OracleAssembler)
    sys.modules[module.__name__] = module
    solvers.solverLibrary["NISTGPU"] = "nonlinearimplicitstaticgpu"
    try:
        U1, its1, R1 = _run_case(case, "NISTGPU", tmp_path)
    finally:
        solvers.solverLibrary.pop("NISTGPU", None)
        sys.modules.pop(module.__name__, None)
    assert its1 == its0
    assert np.abs(U1 - U0).max() <= 1e-9 * np.abs(U0).max()
    assert R1.keys() == R0.keys()
    for name in R0:
        scale = max(np.abs(R0[name]).max(), 1e-300)
        assert np.abs(R1[name] - R0[name]).max() <= 1e-8 * scale, name
