"""Generate Newton-run fixtures by running EdelweissFE simulations with the reference itself.

Usage:  PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_newton_golden.py /path/to/EdelweissFE

For each case (the reference's own edelweiss-provider test inputs under `testfiles/`, plus a few
inputs written here) the script runs `finiteElementSimulation` and records, as arrays:
the mesh (coordinates, per-element type/material/properties/thickness, connectivity, DOF map),
the step's Dirichlet conditions (DOF indices, prescribed values), nodal forces and body forces,
the step controls, every increment the adaptive stepper tried with its Newton iteration count
(or the exception that cut it back), and the converged displacement (plus `U.ref` when present).
"""

import os
import shutil
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import setup_reference  # noqa: E402

CASES = [
    "CantileverBeamQuad4", "CantileverBeamQuad8", "CantileverBeamHexa8", "CantileverBeamVonMisesPE",
    "CantileverBeamQuad8NeoHookeWa", "CantileverBeamQuad8NeoHookeWb", "CantileverBeamQuad8NeoHookeWc",
    "FixedDisplacementQuad4", "FixedDisplacementQuad8", "SimpleBeamHexa8", "SimpleBeamQuad4", "SimpleBeamQuad8",
    "TensionBarHexa8", "TensionBarQuad4", "TensionBarQuad8", "WallShearHexa8", "WallShearHexa20",
]  # fmt: skip

J2_CUBE = """
*material, name=vonmises, id=vonmises, provider=edelweiss
210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0
*job, name=j2job, domain=3d
*solver, solver=NIST, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX={n}
nY={n}
nZ={n}
lX=1
lY=1
lZ=1
elProvider=edelweiss
elType=C3D8
*section, name=section1, material=vonmises, type=solid
all
*step, solver=theSolver, maxInc=0.05, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=off, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 2=0.0
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0
dirichlet, name=back, nSet=gen_back, field=displacement, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=0.005
"""

NH_CUBE = """
*material, name=neohookewa, id=nh, provider=edelweiss
384.6153846, 833.3333333
*job, name=nhjob, domain=3d
*solver, solver=NIST, name=theSolver
*modelGenerator, generator=boxGen, name=gen
nX={n}
nY={n}
nZ={n}
lX=1
lY=1
lZ=1
elProvider=edelweiss
elType=C3D8TL
*section, name=section1, material=nh, type=solid
all
*step, solver=theSolver, maxInc=0.2, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=off, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 1=0.0, 2=0.0, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=-0.05
"""

# a 2x2x2 von Mises cube pulled to 10 % in one increment: a material point of the reference asks for
# a cutback (CutbackRequest) and the stepper retries with a smaller increment.  Recorded under
# golden/newton_cutback/ (the standalone Newton driver's host logic on the CPU).
J2_CUTBACK = """
*material, name=vonmises, id=vonmises, provider=edelweiss
210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0
*job, name=j2job, domain=3d
*solver, solver=NIST, name=theSolver
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
*step, solver=theSolver, maxInc=1.0, minInc=1e-6, maxNumInc=1000, maxIter=25, stepLength=1
options, category=NISTSolver, extrapolation=linear, linsolver=superlu
dirichlet, name=bot, nSet=gen_bottom, field=displacement, 2=0.0
dirichlet, name=left, nSet=gen_left, field=displacement, 1=0.0
dirichlet, name=back, nSet=gen_back, field=displacement, 3=0.0
dirichlet, name=top, nSet=gen_top, field=displacement, 2=0.1
"""


def element_type_name(el):
    from edelweissfe.elements.library import elLibrary

    tl = type(el).__name__ == "DisplacementTLElement"
    for name, v in elLibrary.items():
        if (v["elClass"] == "DisplacementTLElement") != tl:
            continue
        if (
            v["nNodes"] == el.nNodes
            and v["nSpatialDimensions"] == el.nSpatialDimensions
            and v["nInt"] == el._nInt
            and v["plStrain"] == el.planeStrain
            and np.array_equal(v["xi"], el._xi)
        ):
            return name.upper()
    raise KeyError("element type not found")


def material_of(m):
    n = type(m).__name__
    if n == "LinearElasticMaterial":
        return "linearelastic", [m._E, m._v]
    if n == "VonMisesMaterial":
        return "vonmises", [m._E, m._v, m.yieldStress, m.HLin, m.deltaYieldStress, m.delta]
    if n.startswith("NeoHookeanW"):
        return "neohookew" + n[len("NeoHookeanW")].lower(), list(np.asarray(m.materialProperties, float)[:2])
    raise KeyError(n)


def run(name, inp_text, wd, ref_root, subdir="newton"):
    import edelweissfe.solvers.nonlinearimplicitstatic as nis
    from edelweissfe.drivers.inputfiledrivensimulation import finiteElementSimulation
    from edelweissfe.utils.inputfileparser import parseInputFile

    rec = {}
    incs = []
    orig_step, orig_inc = nis.NIST.solveStep, nis.NIST.solveIncrement

    def solve_step(self, step, model, fieldOutputController, outputmanagers):
        rec["solver"] = self
        rec["step"] = step
        rec["model"] = model
        rec["dirichlets"] = list(step.actions["dirichlet"].values())
        rec["nodeforces"] = list(step.actions["nodeforces"].values())
        rec["bodyforces"] = list(step.actions["bodyforce"].values())
        # the step actions reset their increments at the end of the step: copy them now
        rec["dirichlet_values"] = [np.array(d.delta, float).flatten() for d in rec["dirichlets"]]
        rec["nodeforce_values"] = [np.array(f.nodeForcesDelta, float).flatten() for f in rec["nodeforces"]]
        rec["bodyforce_values"] = [np.array(b._delta, float).flatten() for b in rec["bodyforces"]]
        rec["extrapolation"] = self.NISTOptions.get("extrapolation") if hasattr(self, "NISTOptions") else None
        return orig_step(self, step, model, fieldOutputController, outputmanagers)

    def solve_inc(self, U_n, dU, P, K, stepActions, model, timeStep, prevTimeStep, extrapolation, maxIter,
                  maxGrowingIter):  # fmt: skip
        rec.setdefault("extrap_used", extrapolation)
        rec.setdefault("maxIter", maxIter)
        rec.setdefault("maxGrowingIter", maxGrowingIter)
        ts = (timeStep.number, timeStep.stepProgressIncrement, timeStep.stepProgress, timeStep.timeIncrement,
              timeStep.stepTime, timeStep.totalTime)  # fmt: skip
        try:
            out = orig_inc(self, U_n, dU, P, K, stepActions, model, timeStep, prevTimeStep, extrapolation, maxIter,
                           maxGrowingIter)  # fmt: skip
        except Exception as e:
            incs.append(ts + (-1, type(e).__name__))
            raise
        incs.append(ts + (out[3], ""))
        return out

    nis.NIST.solveStep, nis.NIST.solveIncrement = solve_step, solve_inc
    cwd = os.getcwd()
    os.chdir(wd)
    try:
        model, _ = finiteElementSimulation(parseInputFile(inp_text), verbose=False, suppressPlots=True)
    finally:
        os.chdir(cwd)
        nis.NIST.solveStep, nis.NIST.solveIncrement = orig_step, orig_inc
    solver, step = rec["solver"], rec["step"]
    dm = solver.theDofManager
    nodes = list(model.nodes.values())
    pos = {n: i for i, n in enumerate(nodes)}
    elements = list(model.elements.values())
    node_dof = -np.ones(len(nodes), np.int64)
    types_, kinds, props, th, conns = [], [], [], [], []
    for el in elements:
        idx = dm.idcsOfElementsInDofVector[el]
        d = el.nSpatialDimensions
        for a, n in enumerate(el.nodes):
            node_dof[pos[n]] = idx[a * d]
        types_.append(element_type_name(el))
        k, p = material_of(el.material)
        kinds.append(k)
        props.append(p + [0.0] * (6 - len(p)))
        th.append(float(el._t))
        conns.append([pos[n] for n in el.nodes])
    U = np.hstack([f["U"].flatten() for f in model.nodeFields.values()])
    out = dict(
        name=np.array(name),
        coords=np.array([n.coordinates for n in nodes]),
        node_dof=node_dof,
        nDof=np.array(dm.nDof),
        elTypes=np.array(types_),
        kinds=np.array(kinds),
        props=np.array(props),
        thickness=np.array(th),
        conn=np.array(conns, np.int64),
        U_final=U,
        increments=np.array([i[:7] for i in incs], float),
        increment_errors=np.array([i[7] for i in incs]),
        step_controls=np.array([float(step.startIncrementSize), float(step.maxIncrementSize),
                                float(step.minIncrementSize), float(step.maxNumberIncrements), float(step.maxIter),
                                float(step.criticalIter), float(step.maxGrowIter), float(step.cutbackFactor),
                                float(step.length), float(step.incrementGenerator.increaseFactor)]),  # fmt: skip
        extrapolation=np.array(str(rec.get("extrap_used"))),
    )
    for k, d in enumerate(rec["dirichlets"]):
        out[f"dirichlet{k}_dofs"] = solver.findDirichletIndices(d)
        out[f"dirichlet{k}_values"] = rec["dirichlet_values"][k]
    for k, f in enumerate(rec["nodeforces"]):
        out[f"nodeforce{k}_dofs"] = dm.idcsOfFieldsOnNodeSetsInDofVector[f.field][f.nodeSet]
        out[f"nodeforce{k}_values"] = rec["nodeforce_values"][k]
    for k, b in enumerate(rec["bodyforces"]):
        out[f"bodyforce{k}_elements"] = np.array([elements.index(el) for el in b.elementSet], np.int64)
        out[f"bodyforce{k}_values"] = rec["bodyforce_values"][k]
    if os.path.exists(os.path.join(wd, "U.ref")):
        out["U_ref"] = np.loadtxt(os.path.join(wd, "U.ref"))
    os.makedirs(os.path.join(HERE, subdir), exist_ok=True)
    path = os.path.join(HERE, subdir, f"{name}.npz")
    np.savez_compressed(path, **out)
    its = [int(i[6]) for i in incs]
    print(f"{name:32s} el={len(elements):5d} nDof={dm.nDof:6d} incs={len(incs):3d} iters={its}", flush=True)


def main(ref_root, only=None):
    setup_reference(ref_root)
    # the default linear solver (PARDISO) is not available: SuperLU through scipy, as linsolver=superlu
    import scipy.sparse.linalg as sla

    pm = types.ModuleType("edelweissfe.linsolve.pardiso.pardiso")
    pm.pardisoSolve = lambda A, b: sla.spsolve(A, b, use_umfpack=False)
    sys.modules[pm.__name__] = pm
    os.makedirs(os.path.join(HERE, "newton"), exist_ok=True)
    for case in CASES:
        if only and case not in only:
            continue
        wd = tempfile.mkdtemp()
        shutil.copytree(os.path.join(ref_root, "testfiles", case), wd, dirs_exist_ok=True)
        with open(os.path.join(wd, "test.inp")) as f:
            text = f.read()
        inp = os.path.join(wd, "test.inp")
        del text
        from edelweissfe.utils.inputfileparser import parseInputFile  # noqa: F401

        run(case, inp, wd, ref_root)
    written = (("J2Cube6", J2_CUBE.format(n=6), "newton"), ("NeoHookeCube4", NH_CUBE.format(n=4), "newton"),
               ("J2CutbackCube2", J2_CUTBACK, "newton_cutback"))  # fmt: skip
    for name, text, subdir in written:
        if only and name not in only:
            continue
        wd = tempfile.mkdtemp()
        with open(os.path.join(wd, "test.inp"), "w") as f:
            f.write(text)
        run(name, os.path.join(wd, "test.inp"), wd, ref_root, subdir)


if __name__ == "__main__":
    # python make_newton_golden.py /path/to/EdelweissFE [case names: regenerate only those]
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EDELWEISSFE_ROOT", ""), set(sys.argv[2:]) or None)
