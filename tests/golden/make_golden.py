"""Generate golden fixtures by running the EdelweissFE reference itself.

Usage (in a container where the reference source tree is available):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/EdelweissFE

The reference is pure Python/NumPy plus Cython glue.  This script
* compiles `edelweissfe/numerics/csrgenerator.pyx` and
  `edelweissfe/utils/elementresultcollector.pyx` into a temporary directory
  (outside the reference tree) with Cython and loads them under their dotted names;
* stubs the modules the element path imports but does not use
  (the Marmot wrappers imported by `sets/elementset.py:32-35`);
* builds meshes with the reference's own generators, jitters interior nodes,
  re-reads the coordinates with `setNodes`, assigns sections/materials, and
  calls `NIST.computeElements` + `CSRGenerator.updateCSR` in a Newton-like
  sequence of increments and iterations (`acceptLastState` between increments);
* stores inputs and outputs as compressed .npz fixtures next to this script.

The fixtures pin the oracle (and, through it, the CUDA path) to the reference.
"""

import glob
import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def setup_reference(ref_root):
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref_root)
    for name, cls in [
        ("edelweissfe.elements.marmotelement.element", "MarmotElementWrapper"),
        ("edelweissfe.elements.marmotsingleqpelement.element", "MarmotMaterialWrappingElement"),
    ]:
        m = types.ModuleType(name)
        setattr(m, cls, type(cls, (), {}))
        sys.modules[name] = m
    # optional I/O dependencies that are imported at module level but unused on the element path
    from unittest import mock

    for name in ["h5py", "matplotlib", "matplotlib.pyplot", "matplotlib.tri", "matplotlib.colors", "matplotlib.cm",
                 "matplotlib.ticker", "matplotlib.lines", "mpl_toolkits", "mpl_toolkits.mplot3d"]:  # fmt: skip
        if name not in sys.modules:
            try:
                __import__(name)
            except ImportError:
                sys.modules[name] = mock.MagicMock()
    try:
        import prettytable  # noqa: F401
    except ImportError:
        pt = types.ModuleType("prettytable")

        class _PrettyTable:
            def __init__(self, *a, **k):
                self.field_names = []
                self.align = {}

            def add_row(self, *a, **k):
                pass

            def __str__(self):
                return ""

            def get_string(self, *a, **k):
                return ""

        pt.PrettyTable = _PrettyTable
        sys.modules["prettytable"] = pt
    build = tempfile.mkdtemp(prefix="efe_golden_build_")
    modules = {
        "csrgenerator": ("edelweissfe/numerics/csrgenerator.pyx", "edelweissfe.numerics.csrgenerator"),
        "elementresultcollector": (
            "edelweissfe/utils/elementresultcollector.pyx",
            "edelweissfe.utils.elementresultcollector",
        ),
    }
    for short, (rel, _) in modules.items():
        with open(os.path.join(ref_root, rel)) as f:
            text = f.read()
        with open(os.path.join(build, short + ".pyx"), "w") as f:
            f.write(text)
    with open(os.path.join(build, "setup.py"), "w") as f:
        f.write(
            "import numpy\n"
            "from setuptools import setup, Extension\n"
            "from Cython.Build import cythonize\n"
            "ext=[Extension(m,[m+'.pyx'],include_dirs=[numpy.get_include()],language='c++')\n"
            "     for m in ['csrgenerator','elementresultcollector']]\n"
            "setup(ext_modules=cythonize(ext,compiler_directives={'boundscheck':False,'wraparound':False,"
            "'annotation_typing':False},language_level=3))\n"
        )
    cwd = os.getcwd()
    os.chdir(build)
    try:
        rc = os.system(f"{sys.executable} setup.py build_ext --inplace > build.log 2>&1")
        if rc != 0:
            raise RuntimeError("building the Cython modules failed, see " + os.path.join(build, "build.log"))
    finally:
        os.chdir(cwd)
    for short, (_, dotted) in modules.items():
        so = glob.glob(os.path.join(build, short + "*.so"))[0]
        spec = importlib.util.spec_from_file_location(dotted, so)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[spec.name] = mod
        spec.loader.exec_module(mod)


def make_model(dim, generator, gen_lines, elType, jitter, h, seed, lo, hi):
    from edelweissfe.models.femodel import FEModel

    if generator == "planeRectQuad":
        from edelweissfe.generators.planerectquad import generateModelData
    else:
        from edelweissfe.generators.boxgen import generateModelData
    model = FEModel(dim)
    generateModelData(
        {"data": gen_lines + [f"elType={elType}", "elProvider=edelweiss"], "name": "gen"}, model, None
    )
    rng = np.random.default_rng(seed)
    lo = np.asarray(lo, float)
    hi = np.asarray(hi, float)
    for n in model.nodes.values():
        c = n.coordinates
        if np.all(c > lo + 1e-9) and np.all(c < hi - 1e-9):
            n.coordinates[:] = c + rng.uniform(-jitter, jitter, dim) * np.asarray(h)
    for el in model.elements.values():
        el.setNodes(el.nodes)  # re-read the jittered coordinates (element.py:164-175)
    return model


def material_class(kind):
    from edelweissfe.materials.linearelastic.linearelastic import LinearElasticMaterial
    from edelweissfe.materials.neohooke.neohookepencegouformulationa import NeoHookeanWaMaterial
    from edelweissfe.materials.neohooke.neohookepencegouformulationb import NeoHookeanWbMaterial
    from edelweissfe.materials.neohooke.neohookepencegouformulationc import NeoHookeanWcMaterial
    from edelweissfe.materials.vonmises.vonmises import VonMisesMaterial

    return {
        "linearelastic": LinearElasticMaterial,
        "vonmises": VonMisesMaterial,
        "neohookewa": NeoHookeanWaMaterial,
        "neohookewb": NeoHookeanWbMaterial,
        "neohookewc": NeoHookeanWcMaterial,
    }[kind]


def run_case(name, model, elType, kind, props_per_element, thickness, calls, u_scale, seed):
    """Run a Newton-like call sequence through NIST.computeElements + updateCSR and record it."""
    from edelweissfe.config.timing import createTimingDict
    from edelweissfe.journal.journal import Journal
    from edelweissfe.numerics.csrgenerator import CSRGenerator
    from edelweissfe.numerics.dofmanager import DofManager
    from edelweissfe.sets.nodeset import NodeSet
    from edelweissfe.solvers.nonlinearimplicitstatic import NIST
    from edelweissfe.timesteppers.timestep import TimeStep
    from edelweissfe.utils.exceptions import CutbackRequest

    model.nodeSets["all"] = NodeSet("all", list(model.nodes.values()))
    cls = material_class(kind)
    elements = list(model.elements.values())
    for k, el in enumerate(elements):
        el.setProperties(np.array([thickness[k]]))
        el.initializeElement()
        el.setMaterial(cls(np.array(props_per_element[k], float)))
    model._prepareVariablesAndFields(Journal(verbose=False))
    dm = DofManager(model.nodeFields.values(), [], model.elements.values(), [], model.nodeSets.values())
    K = dm.constructVIJSystemMatrix()
    csr = CSRGenerator(K)
    nodes = list(model.nodes.values())
    node_pos = {n: i for i, n in enumerate(nodes)}
    coords = np.array([n.coordinates for n in nodes])
    conn = np.array([[node_pos[n] for n in el.nodes] for el in elements], np.int64)
    el_dofs = np.array([dm.idcsOfElementsInDofVector[el] for el in elements], np.int64)
    node_dof = -np.ones(len(nodes), np.int64)
    for el, dofs in zip(elements, el_dofs):
        d = model.domainSize
        for a, n in enumerate(el.nodes):
            node_dof[node_pos[n]] = dofs[a * d]
    rec = dict(
        name=np.array(name),
        elType=np.array(elType),
        kind=np.array(kind),
        coords=coords,
        conn=conn,
        el_dofs=el_dofs,
        node_dof=node_dof,
        nDof=np.array(dm.nDof),
        props=np.array(props_per_element, float),
        thickness=np.array(thickness, float),
    )
    rng = np.random.default_rng(seed)
    Un = np.zeros(dm.nDof)
    dU = np.zeros(dm.nDof)
    s = types.SimpleNamespace(computationTimes=createTimingDict())
    out = {}
    call = 0
    inc = 0
    for n_iter in calls:
        dU = rng.uniform(-1, 1, dm.nDof) * u_scale
        for it in range(n_iter):
            if it > 0:
                dU = dU + rng.uniform(-1, 1, dm.nDof) * u_scale * 0.1
            U_np = dm.constructDofVector()
            U_np[:] = Un + dU
            dUv = dm.constructDofVector()
            dUv[:] = dU
            P = dm.constructDofVector()
            F = dm.constructDofVector()
            K[:] = 0.0
            ts = TimeStep(inc + 1, 0.1, 0.1 * (inc + 1), 0.1, 0.1 * (inc + 1), 0.1 * (inc + 1))
            raised = -1
            cutback = 0.0
            try:
                P, K, F = NIST.computeElements(s, model.elements, U_np, dUv, P, K, F, ts)
            except CutbackRequest as e:
                # locate the element that raised: first element whose own call raises
                cutback = e.cutbackSize
                for k, el in enumerate(elements):
                    try:
                        el.computeYourself(
                            np.zeros(el.nDof**2), np.zeros(el.nDof), U_np[el], dUv[el], np.zeros(2), 0.1
                        )
                    except CutbackRequest:
                        raised = k
                        break
            out[f"c{call}_U"] = np.array(U_np)
            out[f"c{call}_dU"] = np.array(dUv)
            out[f"c{call}_inc"] = np.array(inc)
            out[f"c{call}_raised"] = np.array(raised)
            out[f"c{call}_cutback"] = np.array(cutback)
            if raised < 0:
                Kc = csr.updateCSR(K)
                out[f"c{call}_P"] = np.array(P)
                out[f"c{call}_F"] = np.array(F)
                if call == 0 or it == n_iter - 1:  # K of the first call and of each increment's last call
                    out[f"c{call}_Kdata"] = Kc.data.copy()
                out[f"c{call}_state"] = np.array([np.array(el._stateVarsTemp) for el in elements])
                if call == 0:
                    rec["indptr"] = Kc.indptr.copy()
                    rec["indices"] = Kc.indices.copy()
            call += 1
            if raised >= 0:
                break
        if raised >= 0:
            break
        for el in elements:  # FEModel.advanceToTime (femodel.py:245-258)
            el.acceptLastState()
        Un = Un + dU
        inc += 1
    rec["n_calls"] = np.array(call)
    rec.update(out)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **rec)
    print(f"{name:28s} nDof={dm.nDof:5d} nnz={len(rec.get('indices', []))} calls={call} -> {os.path.basename(path)}")


def library_fixture():
    from edelweissfe.elements.library import elLibrary

    rec = {}
    for k, v in elLibrary.items():
        key = k.upper()
        rec[f"{key}__meta"] = np.array(
            [v["nNodes"], v["nDof"], v["nSpatialDimensions"], v["nInt"], {True: 1, False: 0, None: -1}[v["plStrain"]]]
        )
        rec[f"{key}__class"] = np.array(v["elClass"])
        rec[f"{key}__xi"] = np.asarray(v["xi"], float)
        rec[f"{key}__eta"] = np.asarray(v["eta"], float)
        if v["zeta"] is not None:
            rec[f"{key}__zeta"] = np.asarray(v["zeta"], float)
        rec[f"{key}__w"] = np.asarray(v["w"], float)
    np.savez_compressed(os.path.join(HERE, "library.npz"), **rec)
    print("library.npz", len(elLibrary), "types")


def geometry_fixture():
    """Reference J, B and nablaN for one distorted element of every shape."""
    import edelweissfe.elements.displacementelement._elementcomputationmatrices as sm
    import edelweissfe.elements.displacementtlelement._elementcomputationmatrices as tm
    from edelweissfe.elements.library import elLibrary

    rng = np.random.default_rng(11)
    ref_nodes = {
        (2, 4): [[0, 0], [1, 0], [1, 1], [0, 1]],
        (2, 8): [[0, 0], [1, 0], [1, 1], [0, 1], [0.5, 0], [1, 0.5], [0.5, 1], [0, 0.5]],
        (3, 8): [[0, 0, 0], [0, 0, 1], [1, 0, 1], [1, 0, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 1, 0]],
        (3, 20): [
            [0, 0, 0], [0, 0, 1], [1, 0, 1], [1, 0, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 1, 0],
            [0, 0, 0.5], [0.5, 0, 1], [1, 0, 0.5], [0.5, 0, 0], [0, 1, 0.5], [0.5, 1, 1], [1, 1, 0.5], [0.5, 1, 0],
            [0, 0.5, 0], [0, 0.5, 1], [1, 0.5, 1], [1, 0.5, 0],
        ],
    }  # fmt: skip
    rec = {}
    for et in ["CPE4", "CPE4R", "CPE4E", "CPE8", "CPE8R", "C3D8", "C3D8R", "C3D8E", "C3D20", "C3D20R"]:
        L = elLibrary[et]
        d, nn = L["nSpatialDimensions"], L["nNodes"]
        X = np.array(ref_nodes[(d, nn)], float) + rng.uniform(-0.12, 0.12, (nn, d))
        rec[f"{et}__X"] = X
        rec[f"{et}__J"] = sm.computeJacobian(L["xi"], L["eta"], L["zeta"], X.T, L["nInt"], nn, d)
        rec[f"{et}__B"] = sm.computeBOperator(L["xi"], L["eta"], L["zeta"], X.T, L["nInt"], nn, d)
        Jt = tm.computeJacobian(L["xi"], L["eta"], L["zeta"], X.T, L["nInt"], nn, d)
        rec[f"{et}__nablaN"] = tm.computeNablaN(L["xi"], L["eta"], L["zeta"], Jt, L["nInt"], nn, d)
        rec[f"{et}__N"] = sm.computeNOperator(L["xi"], L["eta"], L["zeta"], L["nInt"], nn, d)
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **rec)
    print("geometry.npz")


def main(ref_root):
    setup_reference(ref_root)
    library_fixture()
    geometry_fixture()

    LE = [210000.0, 0.3]
    VM = [210000.0, 0.3, 250.0, 1000.0, 0.0, 0.0]
    VMN = [210000.0, 0.3, 355.0, 1000.0, 200.0, 1400.0]  # nonlinear hardening as in CantileverBeamVonMisesPE
    NH = [1000.0, 10000.0]

    def quad(nx, ny, et, seed):
        return make_model(
            2, "planeRectQuad", [f"nX={nx}", f"nY={ny}", "l=1.5", "h=1.0"], et, 0.1, [1.5 / nx, 1.0 / ny], seed,
            [0, 0], [1.5, 1.0]
        )

    def box(nx, ny, nz, et, seed):
        return make_model(
            3, "boxGen", [f"nX={nx}", f"nY={ny}", f"nZ={nz}"], et, 0.1, [1 / nx, 1 / ny, 1 / nz], seed, [0, 0, 0],
            [1, 1, 1]
        )

    # --- config 1: Quad4 plane-strain cantilever 40x8 on [0,10]x[0,2], jitter 10%, LE, one assembly
    m = make_model(2, "planeRectQuad", ["x0=0", "l=10", "y0=0", "h=2", "nX=40", "nY=8"], "CPE4", 0.1,
                   [10 / 40, 2 / 8], 0, [0, 0], [10, 2])  # fmt: skip
    nE = len(m.elements)
    run_case("cfg1_cpe4_le_40x8", m, "CPE4", "linearelastic", [LE] * nE, [1.0] * nE, [1], 1e-3, 0)

    seq = [2, 2]  # iterations per increment
    seed = 100
    for et in ["CPE4", "CPE4R", "CPE4E", "CPE8", "CPE8R", "CPS4", "CPS4R", "CPS4E", "CPS8", "CPS8R"]:
        for kind, props, us in [("linearelastic", LE, 2e-3), ("vonmises", VM, 3e-3), ("vonmises", VMN, 3e-3)]:
            if et.startswith("CPS") and kind == "vonmises":
                us = (1.5e-4 if props is VM else 3e-4) / (3 if "8" in et else 1)  # the reference's plane-stress J2 asks for cutbacks at larger plastic strains
            m = quad(3, 2, et, seed)
            nE = len(m.elements)
            tag = "vmn" if props is VMN else kind[:2]
            run_case(f"ss_{et.lower()}_{tag}", m, et, kind, [props] * nE, [0.8] * nE, seq, us, seed)
            seed += 1
    for et in ["C3D8", "C3D8R", "C3D8E", "C3D20", "C3D20R"]:
        for kind, props, us in [("linearelastic", LE, 2e-3), ("vonmises", VM, 3e-3), ("vonmises", VMN, 3e-3)]:
            m = box(2, 2, 1, et, seed) if "20" not in et else box(2, 1, 1, et, seed)
            nE = len(m.elements)
            tag = "vmn" if props is VMN else kind[:2]
            run_case(f"ss_{et.lower()}_{tag}", m, et, kind, [props] * nE, [1.0] * nE, seq, us, seed)
            seed += 1
    # per-element material parameters (sections with fields, sectionbase.py:86-108)
    m = box(3, 2, 2, "C3D8", seed)
    nE = len(m.elements)
    rng = np.random.default_rng(seed)
    pe = [[210000.0, 0.3, rng.uniform(200, 300), rng.uniform(800, 1200), 0.0, 0.0] for _ in range(nE)]
    run_case("ss_c3d8_vm_perelement", m, "C3D8", "vonmises", pe, [1.0] * nE, seq, 3e-3, seed)
    seed += 1

    for et in ["CPE4TL", "CPE4RTL", "CPE4ETL", "CPE8TL", "CPE8RTL", "C3D8TL", "C3D8RTL", "C3D8ETL", "C3D20TL",
               "C3D20RTL"]:  # fmt: skip
        for kind, props, us in [
            ("neohookewa", NH, 0.03),
            ("neohookewb", NH, 0.03),
            ("neohookewc", NH, 0.03),
            ("linearelastic", LE, 2e-3),
            ("vonmises", VM, 3e-3),
        ]:
            m = quad(3, 2, et, seed) if et.startswith("CP") else box(2, 1 if "20" in et else 2, 1, et, seed)
            nE = len(m.elements)
            run_case(f"tl_{et.lower()}_{kind[:2] if kind[:2] != 'ne' else kind[-2:]}", m, et, kind, [props] * nE,
                     [0.8] * nE, seq, us, seed)  # fmt: skip
            seed += 1
    for et in ["CPS4TL", "CPS8RTL"]:  # plane-stress TL: hypoelastic materials only
        for kind, props, us in [("linearelastic", LE, 2e-3), ("vonmises", VM, 1.5e-4 / (3 if "8" in et else 1))]:
            m = quad(3, 2, et, seed)
            nE = len(m.elements)
            run_case(f"tl_{et.lower()}_{kind[:2]}", m, et, kind, [props] * nE, [0.8] * nE, seq, us, seed)
            seed += 1
    # config-2 shape: Hexa8 J2 3x3x3 jittered 5%, several increments
    m = make_model(3, "boxGen", ["nX=3", "nY=3", "nZ=3"], "C3D8", 0.05, [1 / 3] * 3, 1, [0, 0, 0], [1, 1, 1])
    nE = len(m.elements)
    run_case("cfg2_c3d8_vm_3cube", m, "C3D8", "vonmises", [VM] * nE, [1.0] * nE, [2, 2, 2], 4e-3, 1)
    # plane-stress J2 local Newton that gives up -> CutbackRequest (basehypoelasticmaterial.py:106-109)
    m = quad(3, 2, "CPS4", 8)
    nE = len(m.elements)
    run_case("cutback_cps4_vm", m, "CPS4", "vonmises", [VM] * nE, [0.8] * nE, [1], 3e-3, 8)
    # von Mises return map that stalls on its absolute 1e-12 tolerance -> CutbackRequest
    m = box(1, 1, 1, "C3D20", 7)
    run_case("cutback_c3d20_vm", m, "C3D20", "vonmises", [VM], [1.0], [1], 2e-2, 7)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EDELWEISSFE_ROOT", ""))
