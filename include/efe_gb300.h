/*
 * efe_gb300.h -- C ABI of the GB300 (sm_103a) element-evaluation and CSR-assembly library.
 *
 * The library replaces, for the reference's "edelweiss" displacement elements, the per-element
 * Python loop of NIST.computeElements and the COO->CSR scatter of CSRGenerator.updateCSR:
 *
 *   reference (EdelweissFE, paths relative to the project root)          replaced by
 *   --------------------------------------------------------------------------------------------
 *   solvers/nonlinearimplicitstatic.py:794-849  NIST.computeElements      efe_compute_elements
 *   numerics/csrgenerator.pyx:100-115           CSRGenerator.updateCSR    efe_compute_elements
 *                                                (K is scattered straight into CSR data)
 *   numerics/csrgenerator.pyx:47-98             CSRGenerator.__init__     efe_pattern_count / efe_pattern_fill
 *   numerics/dofmanager.py:522-557              DofManager VIJ pattern    (no VIJ vector is formed)
 *   elements/displacementelement/element.py:194-205 initializeElement     efe_setup_geometry
 *   elements/displacementtlelement/element.py:249-259 initializeElement   efe_setup_geometry
 *   elements/displacementelement/element.py:373-379 acceptLastState      efe_accept_state
 *   elements/displacementtlelement/element.py:454-461 acceptLastState    efe_accept_state
 *   elements/marmotelement/element.pxd:97-103   MarmotElement::computeYourself (native ABI shape:
 *                                                caller-owned buffers, pNewDT status -> CutbackRequest)
 *
 * Conventions
 *   - All array arguments of efe_setup_geometry / efe_compute_elements / efe_accept_state are
 *     DEVICE pointers owned by the caller; the library never allocates on these calls.
 *     efe_pattern_count / efe_pattern_fill work on HOST arrays (set-up, once per mesh).
 *   - `stream` is a cudaStream_t passed as void*; NULL means the legacy default stream.
 *   - Return value 0 = success; otherwise an EFE_ERR_* code, and efe_last_error() describes it.
 *     Numerical failures of material points are never raised on the device: they are reported
 *     in `status` (see EFE_STATUS_*), and the host raises CutbackRequest (utils/exceptions.py:44-49).
 *   - DOF numbering: every node carries `dim` consecutive DOFs starting at nodeDof[node]
 *     (DofManager._reserveSpaceForNodeFields, dofmanager.py:259-300, one displacement field).
 *   - Element matrix placement follows the reference VIJ layout (dofmanager.py:552-554): the
 *     value Ke[(a,j),(b,k)] of element node pair (a,b), components (j,k), is added to the CSR
 *     entry (row = dof(b,k), col = dof(a,j)).
 *   - Per-quadrature-point arrays are structure-of-arrays: field f of point q of element e is at
 *     [f * (nElements * nInt) + e * nInt + q].
 */
#ifndef EFE_GB300_H
#define EFE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EFE_ABI_VERSION 3

/* element shapes (node numbering of computeNOperator, _elementcomputationmatrices.py:106-212) */
enum { EFE_QUAD4 = 0, EFE_QUAD8 = 1, EFE_HEXA8 = 2, EFE_HEXA20 = 3 };
/* quadrature rules of elements/library.py:33-533 */
enum {
  EFE_RULE_2D_1 = 0,     /* 1 point, weight 4                         (CPE4R)          */
  EFE_RULE_2D_2X2 = 1,   /* 2x2 Gauss                                  (CPE4, CPE8R)    */
  EFE_RULE_2D_3X3 = 2,   /* 3x3 Gauss                                  (CPE4E, CPE8)    */
  EFE_RULE_3D_1 = 3,     /* 1 point, weight 8                         (C3D8R)          */
  EFE_RULE_3D_2X2X2 = 4, /* 2x2x2 Gauss                                (C3D8, C3D20R)   */
  EFE_RULE_3D_3X3X3 = 5  /* 3x3x3 Gauss                                (C3D8E, C3D20)   */
};
/* kinematics */
enum { EFE_SMALL_STRAIN = 0, EFE_TOTAL_LAGRANGIAN = 1 };
/* in-plane assumption of 2D elements (library.py plStrain); solids use EFE_SOLID */
enum { EFE_SOLID = 0, EFE_PLANE_STRAIN = 1, EFE_PLANE_STRESS = 2 };
/* materials (edelweissfe/materials): property counts 2, 6, 2, 2, 2 */
enum {
  EFE_MAT_LINEAR_ELASTIC = 0, /* [E, nu]                              linearelastic.py:59-61 */
  EFE_MAT_VON_MISES = 1,      /* [E, nu, fy0, HLin, dfy, delta]       vonmises.py:105-124    */
  EFE_MAT_NEOHOOKE_WA = 2,    /* [mu, K]                              neohookepencegouformulationa.py:65-70 */
  EFE_MAT_NEOHOOKE_WB = 3,
  EFE_MAT_NEOHOOKE_WC = 4
};
/* precision of the assembled tangent (CSR data) */
enum {
  EFE_K_FP64 = 0, /* everything in FP64 (Kdata is double*)                                   */
  EFE_K_FP32 = 1, /* tangent formed and accumulated in FP32 (Kdata is float*); residual, state
                     and the return map stay FP64                                              */
  EFE_K_FP32_FF = 2 /* as EFE_K_FP32, and for small-strain solids the strain increment and the
                     element residual, for total-Lagrangian Neo-Hooke F, F^-T dN/dX and the
                     element residual are formed in float-float arithmetic (~48-bit significand,
                     needs geomG32 and geomGlo); the return map / Kirchhoff stress, state and the
                     global residual accumulation stay FP64                                    */
};
/* status words (int32[3], zeroed by the caller): status[0] = OR of EFE_STATUS_* bits,
   status[1] = INT32_MAX - (global index of the first failing element), 0 if none,
   status[2] = number of failed material points */
enum {
  EFE_STATUS_CUTBACK = 1,      /* a material point asked for a cutback (CutbackRequest(.., 0.5)) */
  EFE_STATUS_BAD_JACOBIAN = 2, /* det J <= 0 or not finite at set-up                               */
  EFE_STATUS_NONFINITE = 4,    /* a non-finite stress was produced                                 */
  EFE_STATUS_TC_TIMEOUT = 8,   /* the tensor-core tangent (tile variant 3) gave up waiting for its
                                  MMAs; K of the pass is incomplete (an internal error)           */
  EFE_STATUS_BOUNDS = 16       /* debug checks (environment EFE_DEVICE_CHECKS=1, read once per
                                  process): a connectivity node outside [0, nNodes), a node DOF
                                  outside the DOF vector, or a pair slot + block offset outside
                                  [0, nnz) in the element pass; the access was skipped, the
                                  pass's outputs are invalid                                     */
};
/* error codes */
enum {
  EFE_OK = 0,
  EFE_ERR_ARGUMENT = 1,
  EFE_ERR_UNSUPPORTED = 2,
  EFE_ERR_CUDA = 3,
  EFE_ERR_PATTERN = 4
};

typedef struct EfeMesh {
  int32_t dim;               /* 2 or 3                                                        */
  int32_t nNodes;            /* number of nodes (including nodes without DOFs)                */
  int64_t nDof;              /* size of the DOF vectors                                      */
  int64_t nnz;               /* number of CSR entries                                        */
  const double* coords;      /* [nNodes][dim] reference coordinates                          */
  const int32_t* nodeDof;    /* [nNodes] first DOF of the node, -1 if it has none            */
  const int32_t* nodeRowLen; /* [nNodes] length of the CSR rows of the node's DOFs           */
} EfeMesh;

typedef struct EfeGroup {
  int32_t shape, rule, kinematics, plane, material, nProps;
  int64_t nElements;
  int64_t elementOffset;     /* global index (element order) of the group's first element   */
  const int32_t* conn;       /* [nElements][nNodes] node indices                              */
  const int32_t* pairSlot;   /* [nElements][nNodes][nNodes]: CSR position of
                                (row = first DOF of node b, col = first DOF of node a)        */
  const double* props;       /* [nElements][nProps] material properties per element          */
  const double* thickness;   /* [nElements] (2D); NULL for solids                            */
  double* geomG;             /* [dim*nNodes][nElements*nInt]  dN_a/dX_c at row c*nNodes+a    */
  float* geomG32;            /* optional FP32 copy of geomG (same layout), read by the FP32
                                tangent of EFE_K_FP32; NULL to convert geomG on the fly      */
  float* geomGlo;            /* optional fl32(geomG - geomG32): geomG32 + geomGlo is geomG in
                                float-float form (EFE_K_FP32_FF)                              */
  double* geomS;             /* [nElements*nInt]  det J * weight * thickness                 */
  double* stateRef;          /* [12 + nMatState][nElements*nInt]  stress(6) strain(6) material;
                                read by efe_compute_elements, written by efe_accept_state      */
  double* stateTemp;         /* same layout, written by efe_compute_elements                 */
  double* auxRef;            /* TL only: Green-Lagrange strain of the last accepted state,
                                [6][nElements*nInt] as (11,22,33,12,23,13); may be NULL for
                                hyperelastic materials                                        */
  double* auxTemp;           /* TL only: Green-Lagrange strain of this call                  */
  int32_t tileVariant;       /* CTA shape of the element pass: 0 = 128 threads, 3 CTAs/SM;
                                1 = 256 threads, larger tiles; 2 = as 0 with 4 CTAs/SM where
                                shared memory allows; 3 = the element tangent on the tensor
                                cores (tcgen05, TF32 hi/lo split, FP32 accumulation in TMEM) for
                                Hexa20 3x3x3 total-Lagrangian Neo-Hooke with an FP32 tangent
                                (EFE_K_FP32 / EFE_K_FP32_FF), otherwise as 0 (chosen by the
                                autotuner)                                                     */
} EfeGroup;

/* One (mesh, group) pair of a persistent launch, with its own DOF vectors and CSR data. */
typedef struct EfeWorkItem {
  const EfeMesh* mesh;
  const EfeGroup* group;
  const double* U;
  const double* dU;
  void* Kdata;
  double* P;
  double* F;
} EfeWorkItem;

int32_t efe_abi_version(void);
const char* efe_last_error(void);

/* Number of material state variables per quadrature point (12 + m). */
int32_t efe_state_size(int32_t material);
/* Number of quadrature points of a rule, nodes of a shape. */
int32_t efe_rule_points(int32_t rule);
int32_t efe_shape_nodes(int32_t shape);

/* Jacobians, dN/dX and det J * w * t of every element and quadrature point (once per mesh);
   status[0] gets EFE_STATUS_BAD_JACOBIAN for det J <= 0. */
int32_t efe_setup_geometry(const EfeMesh* mesh, const EfeGroup* group, int32_t* status, void* stream);

/* One element pass: for every element of every group, material update from stateRef into
   stateTemp, K_e scattered into Kdata (double or float per kPrecision), P_e into P, |P_e| into F.
   U = total displacement (used by total-Lagrangian groups), dU = increment since the last
   accepted state (used by small-strain groups).  P, F and Kdata are accumulated into: the caller
   zeroes them first (nonlinearimplicitstatic.py:419).  time2 = [stepTime, totalTime] (host,
   may be NULL) and dT are accepted for interface parity; the materials here do not use them. */
int32_t efe_compute_elements(const EfeMesh* mesh, const EfeGroup* groups, int32_t nGroups, const double* U,
                             const double* dU, const double* time2, double dT, int32_t kPrecision, void* Kdata,
                             double* P, double* F, int32_t* status, void* stream);

/* Body force of a set of elements of one group, added to P (NIST.computeBodyForces,
   solvers/nonlinearimplicitstatic.py:520-557, element computeBodyForce,
   elements/displacementelement/element.py:348-371 and displacementtlelement/element.py:429-452):
   P[(a,c)] += sum_q N_a(q) * force[c] * detJ_q * w_q * t.  elements: device array of nSelected
   element indices local to the group, or NULL for all nElements; force: HOST array [dim].
   Needs efe_setup_geometry to have run for the group. */
int32_t efe_body_force(const EfeMesh* mesh, const EfeGroup* group, const int32_t* elements, int64_t nSelected,
                       const double* force, double* P, void* stream);

/* Adjoint of the total-Lagrangian hyperelastic element residual (no reference counterpart: the
   reference has no derivatives; this differentiates the residual of
   elements/displacementtlelement/element.py:389-414 with the Neo-Hooke materials of
   materials/neohooke/).  For L = lambda^T P(X, U, mu, K) it adds dL/dX to gX ([nNodes][dim], node
   order of the mesh coordinates) and dL/dmu, dL/dK to gParams ([nElements][2]).  With K lambda =
   dJ/dU (lambda = 0 on prescribed DOFs), these are the gradients dJ/dX and dJ/d(mu, K) of an
   objective J(U) at equilibrium.  U, lambda: device DOF vectors.  Total-Lagrangian groups with
   EFE_MAT_NEOHOOKE_* only. */
int32_t efe_adjoint_tl(const EfeMesh* mesh, const EfeGroup* group, const double* U, const double* lambda, double* gX,
                       double* gParams, void* stream);

/* Reverse mode of one small-strain element pass (no reference counterpart: the reference has no
   derivatives; this differentiates displacementelement/element.py:318-346 with
   linearelastic.py:185-210 and vonmises.py:186-254, the return map through its converged scalar
   equation).  For an increment with state stateBefore ([S][nElements*nInt], the layout of
   stateRef) and DOF increment dU, let the pass produce the new state s (stress, strain, kappa) and
   the residual P.  Given seeds stateBarIn (adjoint of s, same layout; NULL = 0) and Pbar (adjoint
   of P, DOF vector; NULL = 0), it accumulates
     dUbar       += (ds/d dU)^T stateBarIn + (dP/d dU)^T Pbar                 (DOF vector),
     stateBarOut += (ds/d stateBefore)^T stateBarIn + (dP/d stateBefore)^T Pbar (may be NULL),
     gProps      += the same for the material properties, [nElements][nProps] (may be NULL;
                    E, nu for linear elasticity; E, nu, fy0, HLin, dfy, delta for von Mises),
     gX          += the same for the nodal coordinates, [nNodes][dim] in the node order of
                    mesh->coords (may be NULL; through dN/dX and det J, the Hexa20 Jacobian term
                    included).
   With stateBarIn = NULL and Pbar = v, dUbar gets -K v (K the consistent tangent).  Solids, plane
   strain and plane stress (through the reference's local Newton on eps33, iteration by iteration,
   basehypoelasticmaterial.py:71-130); needs efe_setup_geometry (geomG, geomS). */
int32_t efe_adjoint_small_strain(const EfeMesh* mesh, const EfeGroup* group, const double* stateBefore,
                                 const double* dU, const double* Pbar, const double* stateBarIn, double* stateBarOut,
                                 double* dUbar, double* gProps, double* gX, void* stream);

/* The element pass of several groups, possibly of different meshes and dimensions (e.g. batches of
   2D meshes and batches of 3D meshes), in ONE persistent launch: the resident CTAs take tiles of all
   groups from the work counter until all are done (same results as efe_compute_elements on each
   item).  workCounter: one device uint64 of scratch, zeroed by this call.  Implemented for up to
   EFE_PERSISTENT_MAX_GROUPS groups of each of the types Hexa20 3x3x3 and Hexa8 2x2x2 total-
   Lagrangian Neo-Hooke and small-strain von Mises / linear elastic, and Quad8 2x2 total-Lagrangian
   Neo-Hooke, in any order, precision EFE_K_FP64 / EFE_K_FP32 / EFE_K_FP32_FF (the last needs
   geomG32 and geomGlo); with an FP32 tangent and tileVariant 3 on every Hexa20 total-Lagrangian
   group, their tangents run on the tensor cores.  Other types return EFE_ERR_UNSUPPORTED. */
#define EFE_PERSISTENT_MAX_GROUPS 8
int32_t efe_compute_elements_persistent(const EfeWorkItem* items, int32_t nItems, int32_t kPrecision,
                                        uint64_t* workCounter, int32_t* status, void* stream);

/* Allocation-free form of efe_compute_elements_persistent.  No counterpart in the reference: it
   exists for callers that must not allocate device memory -- a host program whose device memory
   belongs to another runtime's pool or arena (a solver framework, a game or simulation engine
   that hands this library pre-sized buffers), or one that cannot afford a cudaMalloc's implicit
   device synchronisation in its time step.  The caller passes the same inputs and outputs
   (work items, status); the work counter lives in a static device array of the library
   (EFE_NOALLOC_SCRATCH_BYTES per GPU that loads the library, held until the process exits)
   instead of a caller-provided buffer.  The call makes no cudaMalloc/cudaFree and calls no
   allocating library routine.
   - The first call on a device looks up the array's device address on that device (with it
     current); make that first call before any stream capture on the device.  The address is
     kept for the life of the process: after cudaDeviceReset on a device (a new primary context)
     this entry point must not be called on that device again.
   - The counter is zeroed by every call, on `stream`, before its launch; status is NOT zeroed
     (the caller zeroes it, as for the other passes).
   - All calls on one device share the array: calls whose launches may overlap on the GPU (other
     streams, other host threads) race on the counter and give wrong results; serialise them.
   - Limit: the counter is 32-bit; a batch whose tile indices (element tiles of both groups plus
     one per resident CTA) exceed EFE_NOALLOC_MAX_TILES is rejected with EFE_ERR_ARGUMENT. */
#define EFE_NOALLOC_SCRATCH_BYTES 256
#define EFE_NOALLOC_MAX_TILES 2147483647LL
int32_t efe_compute_elements_persistent_noalloc(const EfeWorkItem* items, int32_t nItems, int32_t kPrecision,
                                                int32_t* status, void* stream);

/* Linear solve on the device: Jacobi-preconditioned conjugate gradients on the free DOFs of the
   assembled tangent, in place of the reference's direct solve of the Newton correction
   (linearSolve, solvers/nonlinearimplicitstatic.py:727-751: PARDISO, or SciPy's SuperLU on the
   row-modified system of applyDirichletK, :559-593).  The operator is A_ij = K_ij on free rows
   (free_i = 1) and the identity on prescribed rows; K is read as assembled (double or float per
   kPrecision, int32 CSR), products accumulate in FP64.  efe_pcg_start sets x = 0, r = b,
   z = dinv r, p = z for a right-hand side b that is zero on the prescribed DOFs;
   efe_pcg_iterate runs nIterations CG steps (firstIteration = the number already run, whose
   parity selects the scalar buffers); work[2] then holds r.r for the convergence test (one
   small device-to-host read per batch of iterations).  All vectors are caller-owned [n] device
   arrays; work is EFE_PCG_WORK_DOUBLES doubles of caller-owned device scratch. */
#define EFE_PCG_WORK_DOUBLES 6152
typedef struct EfePcg {
  int64_t n;
  const int32_t* indptr;
  const int32_t* indices;
  const void* Kdata;       /* CSR data, double (EFE_K_FP64) or float (EFE_K_FP32, EFE_K_FP32_FF) */
  int32_t kPrecision;
  const uint8_t* freeMask; /* [n] 1 = free DOF, 0 = prescribed; NULL = all free                  */
  const double* dinv;      /* preconditioner: blockSize 1: [n] 1 / K_ii on free DOFs, 1 on
                              prescribed ones; blockSize 2 or 3: [n / bs][bs][bs] inverses of the
                              nodal diagonal blocks (prescribed rows/columns replaced by identity) */
  double* x;
  double* r;
  double* z;
  double* p;
  double* Ap;
  double* work;
  float* pFF;              /* optional [n][2], 8-byte aligned: with FP32 K the CG products run in
                              float-float arithmetic on p = pFF[i][0] + pFF[i][1] (FP32 pipe);
                              NULL: FP64 arithmetic                                            */
  int32_t blockSize;       /* 1, 2 or 3 DOFs per preconditioner block (n a multiple of it)     */
  int32_t patternBlock;    /* 2 or 3: rows come in aligned groups of that many that share one
                              column list (a node's DOF rows; efe_pattern_fill's pattern when
                              every node's first DOF is a multiple of it): the float-float
                              product reads each column index once per group; 0 or 1: none */
} EfePcg;
/* y_i = free_i ? (K x)_i : x_i */
int32_t efe_csr_spmv(const EfePcg* solver, const double* x, double* y, void* stream);
int32_t efe_pcg_start(const EfePcg* solver, const double* b, void* stream);
int32_t efe_pcg_iterate(const EfePcg* solver, int64_t firstIteration, int32_t nIterations, void* stream);

/* Building blocks of a multilevel (aggregation) preconditioner for the same systems; the reference
   reaches multilevel methods only through external solvers behind linearSolve
   (solvers/nonlinearimplicitstatic.py:727-751), so these have no counterpart of their own.
   efe_csr_gemv: y = alpha A x + beta y for an int32 CSR matrix of nRows rows (rectangular allowed:
   the transfer operators between levels); values double or float per kPrecision (EFE_K_FP32 and
   EFE_K_FP32_FF both mean float values here), FP64 arithmetic in a fixed order per row.  With
   freeMask (then nCols == nRows), row r is the identity where freeMask[r] == 0.  beta == 0: y is
   only written.  x and y must not overlap.
   efe_csr_gemv_pairs: the same for float values (EFE_K_FP32 / EFE_K_FP32_FF) with x given as n
   float-float pairs xPairs[i] = (hi, lo), x_i = hi + lo (8-byte aligned): products and row sums in
   float-float arithmetic on the FP32 pipe, ~2^-48 relative to sum |A_ij x_j|.
   efe_chebyshev_step: d = c1 d + c2 dinv r (d not read when c1 == 0), then z += d (accumulate != 0)
   or z = d, for vectors of n doubles: the vector part of one step of a Chebyshev smoother in the
   point-Jacobi-scaled operator; dPairs (optional, 8-byte aligned) receives d as float-float pairs.
   efe_split_pairs: pairs[i] = (fl32(x_i), fl32(x_i - fl32(x_i))). */
typedef struct EfeCsr {
  int64_t nRows;
  int64_t nCols;
  int64_t nnz;             /* indptr[nRows]; rows of at most two entries on average take a
                              one-thread-per-row kernel */
  const int32_t* indptr;   /* [nRows + 1] */
  const int32_t* indices;  /* [nnz], each < nCols */
  const void* values;      /* [nnz] double or float */
  int32_t kPrecision;
  const uint8_t* freeMask; /* [nRows] or NULL */
  int32_t rowBlock;        /* as EfePcg.patternBlock, for efe_csr_gemv_pairs of a square matrix */
} EfeCsr;
int32_t efe_csr_gemv(const EfeCsr* A, const double* x, double alpha, double beta, double* y, void* stream);
int32_t efe_csr_gemv_pairs(const EfeCsr* A, const float* xPairs, double alpha, double beta, double* y, void* stream);
int32_t efe_chebyshev_step(int64_t n, const double* dinv, const double* r, double c1, double c2, int32_t accumulate,
                           double* d, double* z, float* dPairs, void* stream);
int32_t efe_split_pairs(int64_t n, const double* x, float* pairs, void* stream);

/* Measurement aid, no counterpart in the reference: FMA throughput of the FP64 (fp64 != 0) or FP32
   pipe, for the roofline of the element pass, which the FP64 pipe binds on this GPU.  Launches
   `blocks` CTAs of 256 threads, each thread running 8 independent FMA chains of `iterations`
   steps; *flops = the FLOPs of the launch (2 per FMA).  sink: one device double (fp64) or float,
   never written in practice.  The caller times the launch on `stream`. */
int32_t efe_fma_probe(int32_t fp64, int32_t blocks, int64_t iterations, void* sink, void* stream, int64_t* flops);

/* acceptLastState: stateTemp -> stateRef and auxTemp -> auxRef for every group. */
int32_t efe_accept_state(const EfeGroup* groups, int32_t nGroups, void* stream);

/* CSR pattern of the assembled matrix (host arrays; set-up).  conns[g] is [nEl[g]][nNodes[g]].
   efe_pattern_count fills indptr[nDof+1] and nodeRowLen[nNodes] and returns nnz (or -1);
   efe_pattern_fill then fills indices[nnz] (sorted per row, as scipy's canonical CSR) and the
   pair slot maps pairSlots[g] ([nEl[g]][nNodes[g]][nNodes[g]]). */
int64_t efe_pattern_count(int32_t dim, int32_t nNodes, const int32_t* nodeDof, int32_t nGroups,
                          const int32_t* const* conns, const int64_t* nEl, const int32_t* nNodesPerEl,
                          int64_t nDof, int32_t* indptr, int32_t* nodeRowLen);
int32_t efe_pattern_fill(int32_t dim, int32_t nNodes, const int32_t* nodeDof, int32_t nGroups,
                         const int32_t* const* conns, const int64_t* nEl, const int32_t* nNodesPerEl, int64_t nDof,
                         const int32_t* indptr, int32_t* indices, int32_t* const* pairSlots);

#ifdef __cplusplus
}
#endif

#endif /* EFE_GB300_H */
