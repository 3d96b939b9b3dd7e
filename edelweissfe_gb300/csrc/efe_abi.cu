// efe_abi.cu -- extern "C" entry points of libefe_gb300 (declared in include/efe_gb300.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "efe_launch.cuh"

namespace {

thread_local std::string g_last_error;

int32_t fail(int32_t code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int32_t cuda_fail(cudaError_t e, const char* where) {
  return fail(EFE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

int rule_points(int rule) {
  switch (rule) {
    case EFE_RULE_2D_1: return 1;
    case EFE_RULE_2D_2X2: return 4;
    case EFE_RULE_2D_3X3: return 9;
    case EFE_RULE_3D_1: return 1;
    case EFE_RULE_3D_2X2X2: return 8;
    case EFE_RULE_3D_3X3X3: return 27;
  }
  return -1;
}

int shape_nodes(int shape) {
  switch (shape) {
    case EFE_QUAD4: return 4;
    case EFE_QUAD8: return 8;
    case EFE_HEXA8: return 8;
    case EFE_HEXA20: return 20;
  }
  return -1;
}

int shape_dim(int shape) { return (shape == EFE_QUAD4 || shape == EFE_QUAD8) ? 2 : 3; }

bool rule_fits(int shape, int rule) {
  switch (shape) {
    case EFE_QUAD4: return rule == EFE_RULE_2D_1 || rule == EFE_RULE_2D_2X2 || rule == EFE_RULE_2D_3X3;
    case EFE_QUAD8: return rule == EFE_RULE_2D_2X2 || rule == EFE_RULE_2D_3X3;
    case EFE_HEXA8: return rule == EFE_RULE_3D_1 || rule == EFE_RULE_3D_2X2X2 || rule == EFE_RULE_3D_3X3X3;
    case EFE_HEXA20: return rule == EFE_RULE_3D_2X2X2 || rule == EFE_RULE_3D_3X3X3;
  }
  return false;
}

int material_props(int m) {
  switch (m) {
    case EFE_MAT_LINEAR_ELASTIC: return 2;
    case EFE_MAT_VON_MISES: return 6;
    case EFE_MAT_NEOHOOKE_WA:
    case EFE_MAT_NEOHOOKE_WB:
    case EFE_MAT_NEOHOOKE_WC: return 2;
  }
  return -1;
}

bool hyperelastic(int m) {
  return m == EFE_MAT_NEOHOOKE_WA || m == EFE_MAT_NEOHOOKE_WB || m == EFE_MAT_NEOHOOKE_WC;
}

// Row 5 of inv(A) for the Hexa20 polynomial fit of _J3D20
// (displacementelement/_elementcomputationmatrices.py:392-415): A[a][k] = monomial k at node a.
efe::Hexa20Fix hexa20_fix() {
  static const int basis[20][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {0, 1, 1}, {1, 0, 1},
                                   {2, 0, 0}, {0, 2, 0}, {0, 0, 2}, {2, 1, 0}, {1, 2, 0}, {0, 2, 1}, {0, 1, 2},
                                   {1, 0, 2}, {2, 0, 1}, {1, 1, 1}, {2, 1, 1}, {1, 2, 1}, {1, 1, 2}};
  static const int nodes[20][3] = {{-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, 1, 1},
                                   {1, 1, 1},    {1, 1, -1},  {-1, -1, 0}, {0, -1, 1}, {1, -1, 0}, {0, -1, -1},
                                   {-1, 1, 0},   {0, 1, 1},   {1, 1, 0},   {0, 1, -1}, {-1, 0, -1}, {-1, 0, 1},
                                   {1, 0, 1},    {1, 0, -1}};
  double M[20][40];
  for (int a = 0; a < 20; ++a) {
    for (int k = 0; k < 20; ++k) {
      double v = 1.0;
      for (int d = 0; d < 3; ++d)
        for (int p = 0; p < basis[k][d]; ++p) v *= nodes[a][d];
      M[a][k] = v;
    }
    for (int k = 0; k < 20; ++k) M[a][20 + k] = (a == k) ? 1.0 : 0.0;
  }
  for (int c = 0; c < 20; ++c) {  // Gauss-Jordan with partial pivoting
    int piv = c;
    for (int r = c + 1; r < 20; ++r)
      if (std::fabs(M[r][c]) > std::fabs(M[piv][c])) piv = r;
    if (piv != c)
      for (int k = 0; k < 40; ++k) std::swap(M[c][k], M[piv][k]);
    const double d = M[c][c];
    for (int k = 0; k < 40; ++k) M[c][k] /= d;
    for (int r = 0; r < 20; ++r)
      if (r != c) {
        const double f = M[r][c];
        if (f != 0.0)
          for (int k = 0; k < 40; ++k) M[r][k] -= f * M[c][k];
      }
  }
  efe::Hexa20Fix fix;
  for (int a = 0; a < 20; ++a) fix.r[a] = M[5][20 + a];
  return fix;
}

int form_of(const EfeGroup& g) {
  const int dim = shape_dim(g.shape);
  if (g.kinematics == EFE_SMALL_STRAIN) return dim == 3 ? efe::SS3 : efe::SS2;
  if (hyperelastic(g.material)) return efe::TLH;
  return dim == 3 ? efe::TLV3 : efe::TLV2;
}

int32_t check_group(const EfeMesh* mesh, const EfeGroup& g) {
  if (shape_nodes(g.shape) < 0) return fail(EFE_ERR_ARGUMENT, "unknown element shape");
  if (!rule_fits(g.shape, g.rule)) return fail(EFE_ERR_ARGUMENT, "quadrature rule does not match the shape");
  if (shape_dim(g.shape) != mesh->dim) return fail(EFE_ERR_ARGUMENT, "element dimension differs from the mesh");
  if (material_props(g.material) < 0) return fail(EFE_ERR_ARGUMENT, "unknown material");
  if (g.nProps < material_props(g.material)) return fail(EFE_ERR_ARGUMENT, "too few material properties");
  if (g.kinematics != EFE_SMALL_STRAIN && g.kinematics != EFE_TOTAL_LAGRANGIAN)
    return fail(EFE_ERR_ARGUMENT, "unknown kinematics");
  if (g.kinematics == EFE_SMALL_STRAIN && hyperelastic(g.material))
    // displacementelement/element.py:333-334
    return fail(EFE_ERR_UNSUPPORTED,
                "Please use the nonlinear element (displacementtlelement) for hyperelastic materials.");
  if (g.kinematics == EFE_TOTAL_LAGRANGIAN && hyperelastic(g.material) && g.plane == EFE_PLANE_STRESS)
    // materials/base/basehyperelasticmaterial.py:72-95
    return fail(EFE_ERR_UNSUPPORTED, "Plane stress for hyperelastic materials is currently not possible.");
  if (mesh->dim == 2 && g.plane != EFE_PLANE_STRAIN && g.plane != EFE_PLANE_STRESS)
    return fail(EFE_ERR_ARGUMENT, "2D elements need EFE_PLANE_STRAIN or EFE_PLANE_STRESS");
  if (g.nElements < 0) return fail(EFE_ERR_ARGUMENT, "negative element count");
  return EFE_OK;
}

// Device-side bounds checks of the element pass (EFE_STATUS_BOUNDS): on when the environment has
// EFE_DEVICE_CHECKS set to a non-zero integer, read once per process.
int32_t device_checks() {
  static const int32_t on = [] {
    const char* v = std::getenv("EFE_DEVICE_CHECKS");
    return (v && std::atoi(v) != 0) ? 1 : 0;
  }();
  return on;
}

efe::GroupArgs make_args(const EfeMesh* mesh, const EfeGroup& gr, const double* U, const double* dU, void* Kdata,
                         double* P, double* F, int32_t* status) {
  efe::GroupArgs a;
  a.nElements = gr.nElements;
  a.elementOffset = gr.elementOffset;
  a.conn = gr.conn;
  a.pairSlot = gr.pairSlot;
  a.props = gr.props;
  a.thickness = gr.thickness;
  a.geomG = gr.geomG;
  a.geomG32 = gr.geomG32;
  a.geomGlo = gr.geomGlo;
  a.geomS = gr.geomS;
  a.stateRef = gr.stateRef;
  a.stateTemp = gr.stateTemp;
  a.auxRef = gr.auxRef;
  a.auxTemp = gr.auxTemp;
  a.nProps = gr.nProps;
  a.material = gr.material;
  a.plane = gr.plane;
  a.tileVariant = gr.tileVariant;
  a.nodeDof = mesh->nodeDof;
  a.nodeRowLen = mesh->nodeRowLen;
  a.U = U;
  a.dU = dU;
  a.Kdata = Kdata;
  a.P = P;
  a.F = F;
  a.status = status;
  a.nnz = mesh->nnz;
  a.nDof = mesh->nDof;
  a.nNodes = mesh->nNodes;
  a.checks = device_checks();
  return a;
}

int32_t check_item_buffers(const EfeGroup& gr, const double* U, const double* dU) {
  if (gr.nElements == 0) return EFE_OK;  // an empty group touches no buffer
  const bool tl = gr.kinematics == EFE_TOTAL_LAGRANGIAN;
  if (!gr.conn || !gr.pairSlot || !gr.props || !gr.geomG || !gr.geomS || !gr.stateRef || !gr.stateTemp)
    return fail(EFE_ERR_ARGUMENT, "null group buffer");
  if (tl && (!U || !gr.auxTemp)) return fail(EFE_ERR_ARGUMENT, "total-Lagrangian group needs U and auxTemp");
  if (!tl && !dU) return fail(EFE_ERR_ARGUMENT, "small-strain group needs dU");
  return EFE_OK;
}

template <typename F>
void parallel_for(int64_t n, F&& f) {
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (n < 4096) nt = 1;
  std::vector<std::thread> ts;
  const int64_t chunk = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; ++t) {
    const int64_t b = t * chunk, e = std::min<int64_t>(n, b + chunk);
    if (b >= e) break;
    ts.emplace_back([&, b, e] {
      std::vector<int32_t> scratch;
      for (int64_t i = b; i < e; ++i) f(i, scratch);
    });
  }
  for (auto& t : ts) t.join();
}

// node -> (group, element) incidence
struct Incidence {
  std::vector<int64_t> off;
  std::vector<int64_t> items;  // group << 40 | element
};

Incidence incidence(int32_t nNodes, int32_t nGroups, const int32_t* const* conns, const int64_t* nEl,
                    const int32_t* nn) {
  Incidence inc;
  inc.off.assign((size_t)nNodes + 1, 0);
  for (int g = 0; g < nGroups; ++g)
    for (int64_t e = 0; e < nEl[g]; ++e)
      for (int a = 0; a < nn[g]; ++a) inc.off[(size_t)conns[g][e * nn[g] + a] + 1]++;
  for (int32_t n = 0; n < nNodes; ++n) inc.off[n + 1] += inc.off[n];
  inc.items.resize((size_t)inc.off[nNodes]);
  std::vector<int64_t> cur(inc.off.begin(), inc.off.end() - 1);
  for (int g = 0; g < nGroups; ++g)
    for (int64_t e = 0; e < nEl[g]; ++e)
      for (int a = 0; a < nn[g]; ++a) inc.items[(size_t)cur[conns[g][e * nn[g] + a]]++] = ((int64_t)g << 40) | e;
  return inc;
}

// neighbours of node n (nodes sharing an element, with DOFs), sorted by first DOF
void neighbours(int32_t n, const Incidence& inc, const int32_t* const* conns, const int32_t* nn,
                const int32_t* nodeDof, std::vector<int32_t>& out) {
  out.clear();
  for (int64_t k = inc.off[n]; k < inc.off[n + 1]; ++k) {
    const int g = (int)(inc.items[k] >> 40);
    const int64_t e = inc.items[k] & ((int64_t(1) << 40) - 1);
    for (int a = 0; a < nn[g]; ++a) {
      const int32_t m = conns[g][e * nn[g] + a];
      if (nodeDof[m] >= 0) out.push_back(nodeDof[m]);
    }
  }
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
}

}  // namespace

extern "C" {

int32_t efe_abi_version(void) { return EFE_ABI_VERSION; }

const char* efe_last_error(void) { return g_last_error.c_str(); }

int32_t efe_state_size(int32_t material) { return material == EFE_MAT_LINEAR_ELASTIC ? 12 : 13; }

int32_t efe_rule_points(int32_t rule) { return rule_points(rule); }

int32_t efe_shape_nodes(int32_t shape) { return shape_nodes(shape); }

int32_t efe_setup_geometry(const EfeMesh* mesh, const EfeGroup* g, int32_t* status, void* stream) {
  if (!mesh || !g || !status) return fail(EFE_ERR_ARGUMENT, "null argument");
  int32_t rc = check_group(mesh, *g);
  if (rc) return rc;
  if (g->nElements == 0) return EFE_OK;
  if (!g->geomG || !g->geomS || !g->conn || !mesh->coords) return fail(EFE_ERR_ARGUMENT, "null geometry buffer");
  if (mesh->dim == 2 && !g->thickness) return fail(EFE_ERR_ARGUMENT, "2D elements need a thickness array");
  static const efe::Hexa20Fix fix = hexa20_fix();
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaErrorInvalidValue;
  switch (g->shape) {
    case EFE_QUAD4:
      e = efe::geometry_quad4(g->rule, g->nElements, g->elementOffset, g->conn, mesh->coords, g->thickness, g->geomG,
                              g->geomG32, g->geomGlo, g->geomS, status, fix, st);
      break;
    case EFE_QUAD8:
      e = efe::geometry_quad8(g->rule, g->nElements, g->elementOffset, g->conn, mesh->coords, g->thickness, g->geomG,
                              g->geomG32, g->geomGlo, g->geomS, status, fix, st);
      break;
    case EFE_HEXA8:
      e = efe::geometry_hexa8(g->rule, g->nElements, g->elementOffset, g->conn, mesh->coords, nullptr, g->geomG,
                              g->geomG32, g->geomGlo, g->geomS, status, fix, st);
      break;
    case EFE_HEXA20:
      e = efe::geometry_hexa20(g->rule, g->nElements, g->elementOffset, g->conn, mesh->coords, nullptr, g->geomG,
                               g->geomG32, g->geomGlo, g->geomS, status, fix, st);
      break;
  }
  if (e != cudaSuccess) return cuda_fail(e, "efe_setup_geometry");
  return EFE_OK;
}

int32_t efe_compute_elements(const EfeMesh* mesh, const EfeGroup* groups, int32_t nGroups, const double* U,
                             const double* dU, const double* time2, double dT, int32_t kPrecision, void* Kdata,
                             double* P, double* F, int32_t* status, void* stream) {
  (void)time2;
  (void)dT;
  // a model without elements has an empty pattern: K may then be a null pointer
  if (!mesh || !groups || nGroups < 0 || (!Kdata && mesh->nnz > 0) || !P || !F || !status)
    return fail(EFE_ERR_ARGUMENT, "null argument");
  if (kPrecision != EFE_K_FP64 && kPrecision != EFE_K_FP32 && kPrecision != EFE_K_FP32_FF)
    return fail(EFE_ERR_ARGUMENT, "unknown K precision");
  if (!mesh->nodeDof || !mesh->nodeRowLen) return fail(EFE_ERR_ARGUMENT, "mesh without DOF map");
  cudaStream_t st = (cudaStream_t)stream;
  for (int32_t i = 0; i < nGroups; ++i) {
    const EfeGroup& gr = groups[i];
    int32_t rc = check_group(mesh, gr);
    if (rc) return rc;
    if (gr.nElements == 0) continue;
    const bool tl = gr.kinematics == EFE_TOTAL_LAGRANGIAN;
    if (!gr.conn || !gr.pairSlot || !gr.props || !gr.geomG || !gr.geomS || !gr.stateRef || !gr.stateTemp)
      return fail(EFE_ERR_ARGUMENT, "null group buffer");
    if (tl && (!U || !gr.auxTemp)) return fail(EFE_ERR_ARGUMENT, "total-Lagrangian group needs U and auxTemp");
    if (!tl && !dU) return fail(EFE_ERR_ARGUMENT, "small-strain group needs dU");
    if (kPrecision == EFE_K_FP32_FF && (form_of(gr) == efe::SS3 || form_of(gr) == efe::TLH) &&
        (!gr.geomG32 || !gr.geomGlo))
      return fail(EFE_ERR_ARGUMENT, "EFE_K_FP32_FF needs geomG32 and geomGlo");
    const efe::GroupArgs a = make_args(mesh, gr, U, dU, Kdata, P, F, status);
    const int form = form_of(gr);
    cudaError_t e = cudaErrorInvalidValue;
    switch (gr.shape) {
      case EFE_QUAD4: e = efe::assemble_quad4(gr.rule, form, kPrecision, a, st); break;
      case EFE_QUAD8: e = efe::assemble_quad8(gr.rule, form, kPrecision, a, st); break;
      case EFE_HEXA8: e = efe::assemble_hexa8(gr.rule, form, kPrecision, a, st); break;
      case EFE_HEXA20: e = efe::assemble_hexa20(gr.rule, form, kPrecision, a, st); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "efe_compute_elements");
  }
  return EFE_OK;
}

int32_t efe_body_force(const EfeMesh* mesh, const EfeGroup* g, const int32_t* elements, int64_t nSelected,
                       const double* force, double* P, void* stream) {
  if (!mesh || !g || !force || !P || nSelected < 0) return fail(EFE_ERR_ARGUMENT, "null argument");
  int32_t rc = check_group(mesh, *g);
  if (rc) return rc;
  if (!elements) nSelected = g->nElements;
  if (nSelected == 0) return EFE_OK;
  if (!g->geomS || !g->conn || !mesh->nodeDof) return fail(EFE_ERR_ARGUMENT, "group without geometry");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaErrorInvalidValue;
  switch (g->shape) {
    case EFE_QUAD4: e = efe::body_force_quad4(g->rule, nSelected, elements, g->conn, mesh->nodeDof, g->geomS, force, P, st); break;
    case EFE_QUAD8: e = efe::body_force_quad8(g->rule, nSelected, elements, g->conn, mesh->nodeDof, g->geomS, force, P, st); break;
    case EFE_HEXA8: e = efe::body_force_hexa8(g->rule, nSelected, elements, g->conn, mesh->nodeDof, g->geomS, force, P, st); break;
    case EFE_HEXA20: e = efe::body_force_hexa20(g->rule, nSelected, elements, g->conn, mesh->nodeDof, g->geomS, force, P, st); break;
  }
  if (e != cudaSuccess) return cuda_fail(e, "efe_body_force");
  return EFE_OK;
}

int32_t efe_adjoint_tl(const EfeMesh* mesh, const EfeGroup* g, const double* U, const double* lambda, double* gX,
                       double* gParams, void* stream) {
  if (!mesh || !g || !U || !lambda || !gX || !gParams) return fail(EFE_ERR_ARGUMENT, "null argument");
  int32_t rc = check_group(mesh, *g);
  if (rc) return rc;
  if (g->kinematics != EFE_TOTAL_LAGRANGIAN || !hyperelastic(g->material))
    return fail(EFE_ERR_UNSUPPORTED, "the adjoint covers total-Lagrangian Neo-Hooke groups");
  if (g->nElements == 0) return EFE_OK;
  if (!mesh->coords || !mesh->nodeDof || !g->conn || !g->props) return fail(EFE_ERR_ARGUMENT, "null group buffer");
  if (mesh->dim == 2 && !g->thickness) return fail(EFE_ERR_ARGUMENT, "2D elements need a thickness array");
  static const efe::Hexa20Fix fix = hexa20_fix();
  efe::AdjointArgs a{g->nElements, g->conn,      mesh->nodeDof, mesh->coords, U,   lambda, g->props,
                     g->nProps,   g->material,  g->thickness,  fix,          gX,  gParams};
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaErrorInvalidValue;
  switch (g->shape) {
    case EFE_QUAD4: e = efe::adjoint_tl_quad4(g->rule, a, st); break;
    case EFE_QUAD8: e = efe::adjoint_tl_quad8(g->rule, a, st); break;
    case EFE_HEXA8: e = efe::adjoint_tl_hexa8(g->rule, a, st); break;
    case EFE_HEXA20: e = efe::adjoint_tl_hexa20(g->rule, a, st); break;
  }
  if (e != cudaSuccess) return cuda_fail(e, "efe_adjoint_tl");
  return EFE_OK;
}

int32_t efe_adjoint_small_strain(const EfeMesh* mesh, const EfeGroup* g, const double* stateBefore, const double* dU,
                                 const double* Pbar, const double* stateBarIn, double* stateBarOut, double* dUbar,
                                 double* gProps, double* gX, void* stream) {
  if (!mesh || !g || !stateBefore || !dU || !dUbar) return fail(EFE_ERR_ARGUMENT, "null argument");
  int32_t rc = check_group(mesh, *g);
  if (rc) return rc;
  if (g->kinematics != EFE_SMALL_STRAIN)
    return fail(EFE_ERR_UNSUPPORTED, "efe_adjoint_small_strain covers small-strain groups");
  if (g->material != EFE_MAT_LINEAR_ELASTIC && g->material != EFE_MAT_VON_MISES)
    return fail(EFE_ERR_UNSUPPORTED, "efe_adjoint_small_strain covers linear elastic and von Mises groups");
  if (g->nElements == 0) return EFE_OK;
  if (!mesh->nodeDof || !g->conn || !g->props || !g->geomG || !g->geomS)
    return fail(EFE_ERR_ARGUMENT, "null group buffer (has efe_setup_geometry run?)");
  efe::SSAdjointArgs a;
  a.nEl = g->nElements;
  a.nProps = g->nProps;
  a.material = g->material;
  a.planeStress = mesh->dim == 2 && g->plane == EFE_PLANE_STRESS;
  a.conn = g->conn;
  a.nodeDof = mesh->nodeDof;
  a.props = g->props;
  a.geomG = g->geomG;
  a.geomG32 = g->geomG32;
  a.geomGlo = g->geomGlo;
  a.geomS = g->geomS;
  a.stateBefore = stateBefore;
  a.dU = dU;
  a.Pbar = Pbar;
  a.barIn = stateBarIn;
  a.barOut = stateBarOut;
  a.dUbar = dUbar;
  a.gProps = gProps;
  a.gX = gX;
  a.coords = mesh->coords;
  if (gX && !mesh->coords) return fail(EFE_ERR_ARGUMENT, "coordinate adjoints need the mesh coordinates");
  static const efe::Hexa20Fix fix = hexa20_fix();
  a.fix = fix;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaErrorInvalidValue;
  switch (g->shape) {
    case EFE_QUAD4: e = efe::adjoint_ss_quad4(g->rule, a, st); break;
    case EFE_QUAD8: e = efe::adjoint_ss_quad8(g->rule, a, st); break;
    case EFE_HEXA8: e = efe::adjoint_ss_hexa8(g->rule, a, st); break;
    case EFE_HEXA20: e = efe::adjoint_ss_hexa20(g->rule, a, st); break;
  }
  if (e != cudaSuccess) return cuda_fail(e, "efe_adjoint_small_strain");
  return EFE_OK;
}

namespace {
// The work items of a persistent pass, sorted by element type (efe::persistent_type_index).
struct PersistentItems {
  efe::GroupArgs g[efe::PERSISTENT_NTYPES][efe::MAX_PERSISTENT_GROUPS];
  int n[efe::PERSISTENT_NTYPES] = {};
};

int32_t persistent_items(const EfeWorkItem* items, int32_t nItems, int32_t kPrecision, int32_t* status,
                         PersistentItems& out) {
  if (!items || nItems < 1 || !status) return fail(EFE_ERR_ARGUMENT, "work items and a status word expected");
  if (kPrecision != EFE_K_FP64 && kPrecision != EFE_K_FP32 && kPrecision != EFE_K_FP32_FF)
    return fail(EFE_ERR_ARGUMENT, "unknown K precision");
  for (int32_t i = 0; i < nItems; ++i) {
    const EfeWorkItem& it = items[i];
    if (!it.mesh || !it.group || !it.P || !it.F || (!it.Kdata && it.mesh->nnz > 0))
      return fail(EFE_ERR_ARGUMENT, "null work item buffer");
    int32_t rc = check_group(it.mesh, *it.group);
    if (rc) return rc;
    rc = check_item_buffers(*it.group, it.U, it.dU);
    if (rc) return rc;
    const EfeGroup& g = *it.group;
    // every type of the persistent kernels has a float-float form (small strain 3D, TL Neo-Hooke)
    if (kPrecision == EFE_K_FP32_FF && g.nElements > 0 && (!g.geomG32 || !g.geomGlo))
      return fail(EFE_ERR_ARGUMENT, "EFE_K_FP32_FF needs geomG32 and geomGlo");
    const int type = efe::persistent_type_index(g.shape, g.rule, form_of(g));
    if (type < 0)
      return fail(EFE_ERR_UNSUPPORTED,
                  "no persistent kernel for this element type (implemented: Hexa20 3x3x3 and Hexa8 2x2x2 total-"
                  "Lagrangian Neo-Hooke and small-strain von Mises / linear elastic, Quad8 2x2 total-Lagrangian "
                  "Neo-Hooke)");
    int& n = out.n[type];
    if (n == efe::MAX_PERSISTENT_GROUPS)
      return fail(EFE_ERR_ARGUMENT, "at most " + std::to_string(efe::MAX_PERSISTENT_GROUPS) +
                                        " groups of each element type in one persistent pass");
    out.g[type][n++] = make_args(it.mesh, g, it.U, it.dU, it.Kdata, it.P, it.F, status);
  }
  return EFE_OK;
}
}  // namespace

int32_t efe_compute_elements_persistent(const EfeWorkItem* items, int32_t nItems, int32_t kPrecision,
                                        uint64_t* workCounter, int32_t* status, void* stream) {
  if (!workCounter) return fail(EFE_ERR_ARGUMENT, "null work counter");
  PersistentItems pi;
  int32_t rc = persistent_items(items, nItems, kPrecision, status, pi);
  if (rc) return rc;
  cudaError_t e = efe::persistent_groups(kPrecision, pi.g, pi.n, (unsigned long long*)workCounter,
                                         (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_compute_elements_persistent");
  return EFE_OK;
}

// Same validation and kernels as efe_compute_elements_persistent; the work counter comes from the
// library's static scratch array (efe_batch.cu), so nothing here allocates device memory.
int32_t efe_compute_elements_persistent_noalloc(const EfeWorkItem* items, int32_t nItems, int32_t kPrecision,
                                                int32_t* status, void* stream) {
  PersistentItems pi;
  int32_t rc = persistent_items(items, nItems, kPrecision, status, pi);
  if (rc) return rc;
  int64_t needed = 0;
  cudaError_t e = efe::persistent_groups_noalloc(kPrecision, pi.g, pi.n, &needed, (cudaStream_t)stream);
  if (needed > EFE_NOALLOC_MAX_TILES) {
    return fail(EFE_ERR_ARGUMENT, "efe_compute_elements_persistent_noalloc: the batch needs " + std::to_string(needed) +
                                      " tile indices, the 32-bit work counter in the static scratch allows at most " +
                                      std::to_string((long long)EFE_NOALLOC_MAX_TILES) +
                                      "; split the batch or use efe_compute_elements_persistent");
  }
  if (e != cudaSuccess) return cuda_fail(e, "efe_compute_elements_persistent_noalloc");
  return EFE_OK;
}

namespace {
int32_t check_pcg(const EfePcg* s) {
  if (!s) return fail(EFE_ERR_ARGUMENT, "null solver");
  if (s->n < 0) return fail(EFE_ERR_ARGUMENT, "negative system size");
  if (s->kPrecision != EFE_K_FP64 && s->kPrecision != EFE_K_FP32 && s->kPrecision != EFE_K_FP32_FF)
    return fail(EFE_ERR_ARGUMENT, "unknown K precision");
  if (s->n > 0 && (!s->indptr || !s->indices || !s->Kdata || !s->dinv || !s->x || !s->r || !s->z || !s->p ||
                   !s->Ap || !s->work))
    return fail(EFE_ERR_ARGUMENT, "null solver buffer");
  if (reinterpret_cast<uintptr_t>(s->pFF) % 8 != 0) return fail(EFE_ERR_ARGUMENT, "pFF must be 8-byte aligned");
  if (s->patternBlock < 0 || s->patternBlock > 3) return fail(EFE_ERR_ARGUMENT, "patternBlock must be 0 to 3");
  if (s->blockSize < 1 || s->blockSize > 3 || s->n % s->blockSize != 0)
    return fail(EFE_ERR_ARGUMENT, "blockSize must be 1, 2 or 3 and divide n");
  return EFE_OK;
}
}  // namespace

int32_t efe_csr_spmv(const EfePcg* s, const double* x, double* y, void* stream) {
  int32_t rc = check_pcg(s);
  if (rc) return rc;
  if (s->n > 0 && (!x || !y)) return fail(EFE_ERR_ARGUMENT, "null vector");
  cudaError_t e = efe::csr_spmv(*s, x, y, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_csr_spmv");
  return EFE_OK;
}

int32_t efe_pcg_start(const EfePcg* s, const double* b, void* stream) {
  int32_t rc = check_pcg(s);
  if (rc) return rc;
  if (s->n > 0 && !b) return fail(EFE_ERR_ARGUMENT, "null right-hand side");
  if (s->n == 0) return EFE_OK;
  cudaError_t e = efe::pcg_start(*s, b, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_pcg_start");
  return EFE_OK;
}

int32_t efe_csr_gemv(const EfeCsr* a, const double* x, double alpha, double beta, double* y, void* stream) {
  if (!a) return fail(EFE_ERR_ARGUMENT, "null matrix");
  if (a->nRows < 0 || a->nCols < 0 || a->nnz < 0) return fail(EFE_ERR_ARGUMENT, "negative matrix size");
  if (a->kPrecision != EFE_K_FP64 && a->kPrecision != EFE_K_FP32 && a->kPrecision != EFE_K_FP32_FF)
    return fail(EFE_ERR_ARGUMENT, "unknown value precision");
  if (a->freeMask && a->nCols != a->nRows) return fail(EFE_ERR_ARGUMENT, "a masked matrix must be square");
  if (a->nRows == 0) return EFE_OK;
  if (!a->indptr || (a->nCols > 0 && (!a->indices || !a->values)) || !y || (a->nCols > 0 && !x))
    return fail(EFE_ERR_ARGUMENT, "null matrix or vector");
  cudaError_t e = efe::csr_gemv(*a, x, alpha, beta, y, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_csr_gemv");
  return EFE_OK;
}

int32_t efe_csr_gemv_pairs(const EfeCsr* a, const float* xPairs, double alpha, double beta, double* y,
                           void* stream) {
  if (!a) return fail(EFE_ERR_ARGUMENT, "null matrix");
  if (a->nRows < 0 || a->nCols < 0 || a->nnz < 0) return fail(EFE_ERR_ARGUMENT, "negative matrix size");
  if (a->kPrecision != EFE_K_FP32 && a->kPrecision != EFE_K_FP32_FF)
    return fail(EFE_ERR_ARGUMENT, "float-float products need float values");
  if (a->rowBlock < 0 || a->rowBlock > 3) return fail(EFE_ERR_ARGUMENT, "rowBlock must be 0 to 3");
  if (a->freeMask && a->nCols != a->nRows) return fail(EFE_ERR_ARGUMENT, "a masked matrix must be square");
  if (reinterpret_cast<uintptr_t>(xPairs) % 8 != 0) return fail(EFE_ERR_ARGUMENT, "xPairs must be 8-byte aligned");
  if (a->nRows == 0) return EFE_OK;
  if (!a->indptr || (a->nCols > 0 && (!a->indices || !a->values || !xPairs)) || !y)
    return fail(EFE_ERR_ARGUMENT, "null matrix or vector");
  cudaError_t e = efe::csr_gemv_pairs(*a, reinterpret_cast<const float2*>(xPairs), alpha, beta, y,
                                      (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_csr_gemv_pairs");
  return EFE_OK;
}

int32_t efe_chebyshev_step(int64_t n, const double* dinv, const double* r, double c1, double c2, int32_t accumulate,
                           double* d, double* z, float* dPairs, void* stream) {
  if (n < 0) return fail(EFE_ERR_ARGUMENT, "negative vector size");
  if (reinterpret_cast<uintptr_t>(dPairs) % 8 != 0) return fail(EFE_ERR_ARGUMENT, "dPairs must be 8-byte aligned");
  if (n == 0) return EFE_OK;
  if (!dinv || !r || !d || !z) return fail(EFE_ERR_ARGUMENT, "null vector");
  cudaError_t e = efe::chebyshev_step(n, dinv, r, c1, c2, accumulate, d, z, reinterpret_cast<float2*>(dPairs),
                                      (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_chebyshev_step");
  return EFE_OK;
}

int32_t efe_split_pairs(int64_t n, const double* x, float* pairs, void* stream) {
  if (n < 0) return fail(EFE_ERR_ARGUMENT, "negative vector size");
  if (reinterpret_cast<uintptr_t>(pairs) % 8 != 0) return fail(EFE_ERR_ARGUMENT, "pairs must be 8-byte aligned");
  if (n == 0) return EFE_OK;
  if (!x || !pairs) return fail(EFE_ERR_ARGUMENT, "null vector");
  cudaError_t e = efe::split_pairs(n, x, reinterpret_cast<float2*>(pairs), (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_split_pairs");
  return EFE_OK;
}

int32_t efe_pcg_iterate(const EfePcg* s, int64_t firstIteration, int32_t nIterations, void* stream) {
  int32_t rc = check_pcg(s);
  if (rc) return rc;
  if (firstIteration < 0 || nIterations < 0) return fail(EFE_ERR_ARGUMENT, "negative iteration count");
  if (s->n == 0) return EFE_OK;
  cudaError_t e = efe::pcg_iterate(*s, firstIteration, nIterations, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_pcg_iterate");
  return EFE_OK;
}

int32_t efe_fma_probe(int32_t fp64, int32_t blocks, int64_t iterations, void* sink, void* stream,
                      int64_t* flops) {
  if (blocks < 1 || iterations < 0 || !sink || !flops) return fail(EFE_ERR_ARGUMENT, "efe_fma_probe: bad argument");
  *flops = efe::fma_probe_flops(blocks, iterations);
  cudaError_t e = efe::fma_probe(fp64, blocks, iterations, sink, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "efe_fma_probe");
  return EFE_OK;
}

int32_t efe_accept_state(const EfeGroup* groups, int32_t nGroups, void* stream) {
  if (!groups || nGroups < 0) return fail(EFE_ERR_ARGUMENT, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  for (int32_t i = 0; i < nGroups; ++i) {
    const EfeGroup& g = groups[i];
    const int nq = rule_points(g.rule);
    if (nq < 0) return fail(EFE_ERR_ARGUMENT, "unknown quadrature rule");
    const size_t n = (size_t)g.nElements * nq;
    if (n == 0) continue;
    const size_t bytes = sizeof(double) * n * efe_state_size(g.material);
    cudaError_t e = cudaMemcpyAsync(g.stateRef, g.stateTemp, bytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "efe_accept_state");
    if (g.kinematics == EFE_TOTAL_LAGRANGIAN && g.auxRef && g.auxTemp) {
      e = cudaMemcpyAsync(g.auxRef, g.auxTemp, sizeof(double) * n * 6, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return cuda_fail(e, "efe_accept_state");
    }
  }
  return EFE_OK;
}

int64_t efe_pattern_count(int32_t dim, int32_t nNodes, const int32_t* nodeDof, int32_t nGroups,
                          const int32_t* const* conns, const int64_t* nEl, const int32_t* nn, int64_t nDof,
                          int32_t* indptr, int32_t* nodeRowLen) {
  if (dim < 1 || nNodes < 0 || !nodeDof || !conns || !nEl || !nn || !indptr || !nodeRowLen) {
    fail(EFE_ERR_ARGUMENT, "null argument");
    return -1;
  }
  for (int32_t n = 0; n < nNodes; ++n)
    if (nodeDof[n] >= 0 && (nodeDof[n] + dim > nDof)) {
      fail(EFE_ERR_PATTERN, "node DOF outside the DOF vector");
      return -1;
    }
  const Incidence inc = incidence(nNodes, nGroups, conns, nEl, nn);
  std::vector<int64_t> rowlen((size_t)nDof, 0);
  parallel_for(nNodes, [&](int64_t n, std::vector<int32_t>& nb) {
    if (nodeDof[n] < 0) {
      nodeRowLen[n] = 0;
      return;
    }
    neighbours((int32_t)n, inc, conns, nn, nodeDof, nb);
    nodeRowLen[n] = (int32_t)(dim * nb.size());
    for (int c = 0; c < dim; ++c) rowlen[(size_t)nodeDof[n] + c] = nodeRowLen[n];
  });
  int64_t acc = 0;
  indptr[0] = 0;
  for (int64_t r = 0; r < nDof; ++r) {
    acc += rowlen[(size_t)r];
    if (acc > INT32_MAX) {
      fail(EFE_ERR_PATTERN, "more than 2^31-1 CSR entries (int32 indices, as scipy's CSR of the reference)");
      return -1;
    }
    indptr[r + 1] = (int32_t)acc;
  }
  return acc;
}

int32_t efe_pattern_fill(int32_t dim, int32_t nNodes, const int32_t* nodeDof, int32_t nGroups,
                         const int32_t* const* conns, const int64_t* nEl, const int32_t* nn, int64_t nDof,
                         const int32_t* indptr, int32_t* indices, int32_t* const* pairSlots) {
  if (dim < 1 || nNodes < 0 || !nodeDof || !conns || !nEl || !nn || !indptr || !indices)
    return fail(EFE_ERR_ARGUMENT, "null argument");
  (void)nDof;
  const Incidence inc = incidence(nNodes, nGroups, conns, nEl, nn);
  parallel_for(nNodes, [&](int64_t n, std::vector<int32_t>& nb) {
    if (nodeDof[n] < 0) return;
    neighbours((int32_t)n, inc, conns, nn, nodeDof, nb);
    for (int c = 0; c < dim; ++c) {
      int32_t* row = indices + indptr[nodeDof[n] + c];
      for (size_t k = 0; k < nb.size(); ++k)
        for (int j = 0; j < dim; ++j) row[k * dim + j] = nb[k] + j;
    }
  });
  if (pairSlots) {
    std::atomic<int32_t> bad{0};  // set by any of the parallel_for threads
    for (int g = 0; g < nGroups; ++g) {
      if (!pairSlots[g]) continue;
      const int32_t* conn = conns[g];
      const int m = nn[g];
      int32_t* slots = pairSlots[g];
      parallel_for(nEl[g], [&](int64_t e, std::vector<int32_t>&) {
        for (int a = 0; a < m; ++a)
          for (int b = 0; b < m; ++b) {
            // CSR position of (row = first DOF of node b, col = first DOF of node a)
            const int32_t rowDof = nodeDof[conn[e * m + b]], colDof = nodeDof[conn[e * m + a]];
            const int32_t* beg = indices + indptr[rowDof];
            const int32_t* end = indices + indptr[rowDof + 1];
            const int32_t* it = std::lower_bound(beg, end, colDof);
            if (it == end || *it != colDof) {
              bad.store(1, std::memory_order_relaxed);
              slots[(e * m + a) * m + b] = -1;
            } else {
              slots[(e * m + a) * m + b] = (int32_t)(it - indices);
            }
          }
      });
    }
    if (bad.load()) return fail(EFE_ERR_PATTERN, "element node pair missing from the pattern");
  }
  return EFE_OK;
}

}  // extern "C"
