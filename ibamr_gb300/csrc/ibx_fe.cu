// ibx_fe.cu -- the finite-element quadrature-point path of FEDataManager on
// the device (ibx_fe_quadrature_points, ibx_fe_assemble_rhs in
// include/ibx.h), for first-order Lagrange simplices: TRI3 in 2D, TET4 in 3D.
//
// FEDataManager::spread (ibtk/src/lagrangian/FEDataManager.cpp:1088-1219)
// evaluates, at every quadrature point q of every element, the position
// X_q = sum_k X_k phi_k(q) and the force density times the quadrature weight
// F_q = (sum_k F_k phi_k(q)) * JxW(q) (sum_weighted_elem_solution,
// FEDataManager.cpp:824-858: the sums start from zero and run over the basis
// functions in order), and spreads F_q from X_q through the raw-array
// LEInteractor::spread.  FEDataManager::interp (FEDataManager.cpp:1873-2005)
// interpolates the Eulerian field at the quadrature points through the
// raw-array LEInteractor::interpolate and assembles the right-hand side of
// the L2 projection, rhs_k += sum_q U_q * (phi_k(q) * JxW(q)) per element
// (integrate_elem_rhs, FEDataManager.cpp:1569-1604).  Two element families
// of first-order Lagrange elements:
//  - simplices (TRI3, TET4): the barycentric basis (phi_0 = 1 - sum_d xi_d,
//    phi_d = xi_d) and JxW(q) = |det J| * w(q) with J the constant Jacobian
//    [X_1 - X_0, ...];
//  - tensor-product cells (QUAD4, HEX8) on the reference cell [-1, 1]^dim,
//    libMesh's node order (counter-clockwise in each z layer, the z = -1
//    layer first): phi_k = L_{a_k}(xi) L_{b_k}(eta) [L_{c_k}(zeta)] with
//    L_0(t) = (1 - t) / 2, L_1(t) = (1 + t) / 2, and JxW(q) = |det J(q)| w(q)
//    with J(q)_{rc} = sum_k X_k[r] dphi_k/dxi_c (q), summed in node order.
// Every product and sum is rounded explicitly, in the order written, so the
// values are those of a sequential evaluation.

#include "ibx_internal.h"
#include "../../include/ibx.h"

#include <cmath>

namespace ibx
{
namespace
{
constexpr int FE_MAX_QP = 64;
constexpr int FE_MAX_NODES = 8;

struct FeRule
{
    int n_qp;
    double phi[FE_MAX_QP][FE_MAX_NODES];     // phi_k at each point
    double dphi[FE_MAX_QP][FE_MAX_NODES][3]; // dphi_k / dxi_c (tensor-product cells)
    double w[FE_MAX_QP];                     // reference weights
};

// Nodes per element of a family.
__host__ __device__ constexpr int
fe_nodes(int dim, int type)
{
    return type == IBX_FE_TENSOR_Q1 ? (dim == 2 ? 4 : 8) : dim + 1;
}

// |det J(q)| of a tensor-product cell: J_rc = sum_k X_k[r] dphi_k/dxi_c.
template <int DIM>
__device__ __forceinline__ double
abs_det_q1(const double* X, const int* nodes, const FeRule& R, int q)
{
    constexpr int NPE = DIM == 2 ? 4 : 8;
    double J[3][3];
    for (int r = 0; r < DIM; ++r)
        for (int c = 0; c < DIM; ++c)
        {
            double v = 0.0;
            for (int k = 0; k < NPE; ++k)
                v = __dadd_rn(v, __dmul_rn(X[(long long)DIM * nodes[k] + r], R.dphi[q][k][c]));
            J[r][c] = v;
        }
    double det;
    if (DIM == 2)
        det = __dsub_rn(__dmul_rn(J[0][0], J[1][1]), __dmul_rn(J[0][1], J[1][0]));
    else
    {
        const double m0 = __dsub_rn(__dmul_rn(J[1][1], J[2][2]), __dmul_rn(J[1][2], J[2][1]));
        const double m1 = __dsub_rn(__dmul_rn(J[1][0], J[2][2]), __dmul_rn(J[1][2], J[2][0]));
        const double m2 = __dsub_rn(__dmul_rn(J[1][0], J[2][1]), __dmul_rn(J[1][1], J[2][0]));
        det = __dadd_rn(__dsub_rn(__dmul_rn(J[0][0], m0), __dmul_rn(J[0][1], m1)), __dmul_rn(J[0][2], m2));
    }
    return fabs(det);
}

// |det J| of element e (columns X_k - X_0).
template <int DIM>
__device__ __forceinline__ double
abs_det(const double* X, const int* nodes)
{
    double J[3][3];
    for (int c = 0; c < DIM; ++c)
        for (int r = 0; r < DIM; ++r)
            J[r][c] = __dsub_rn(X[(long long)DIM * nodes[c + 1] + r], X[(long long)DIM * nodes[0] + r]);
    double det;
    if (DIM == 2)
        det = __dsub_rn(__dmul_rn(J[0][0], J[1][1]), __dmul_rn(J[0][1], J[1][0]));
    else
    {
        const double m0 = __dsub_rn(__dmul_rn(J[1][1], J[2][2]), __dmul_rn(J[1][2], J[2][1]));
        const double m1 = __dsub_rn(__dmul_rn(J[1][0], J[2][2]), __dmul_rn(J[1][2], J[2][0]));
        const double m2 = __dsub_rn(__dmul_rn(J[1][0], J[2][1]), __dmul_rn(J[1][1], J[2][0]));
        det = __dadd_rn(__dsub_rn(__dmul_rn(J[0][0], m0), __dmul_rn(J[0][1], m1)), __dmul_rn(J[0][2], m2));
    }
    return fabs(det);
}

// JxW(q) of an element of the family TYPE.
template <int DIM, int TYPE>
__device__ __forceinline__ double
elem_jxw(const double* X, const int* nodes, const FeRule& R, int q)
{
    const double det = TYPE == IBX_FE_TENSOR_Q1 ? abs_det_q1<DIM>(X, nodes, R, q) : abs_det<DIM>(X, nodes);
    return __dmul_rn(det, R.w[q]);
}

// One thread per (element, quadrature point).
template <int DIM, int TYPE>
__global__ void
fe_qp_kernel(int n_elems, const int* elem_nodes, const double* X, const FeRule R, const double* F, int n_vars,
             double* X_qp, double* F_qp, double* JxW_out, int* status)
{
    constexpr int NPE = fe_nodes(DIM, TYPE);
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n_elems * R.n_qp) return;
    const int e = (int)(t / R.n_qp), q = (int)(t % R.n_qp);
    const int* nodes = elem_nodes + (long long)NPE * e;
    for (int k = 0; k < NPE; ++k)
        if (nodes[k] < 0)
        {
            atomicOr(status, 1);
            return;
        }
    for (int d = 0; d < DIM; ++d)
    {
        double v = 0.0;
        for (int k = 0; k < NPE; ++k) v = __dadd_rn(v, __dmul_rn(X[(long long)DIM * nodes[k] + d], R.phi[q][k]));
        if (X_qp) X_qp[(long long)DIM * t + d] = v;
    }
    const double jxw = elem_jxw<DIM, TYPE>(X, nodes, R, q);
    if (JxW_out) JxW_out[t] = jxw;
    if (F && F_qp)
        for (int i = 0; i < n_vars; ++i)
        {
            double v = 0.0;
            for (int k = 0; k < NPE; ++k)
                v = __dadd_rn(v, __dmul_rn(F[(long long)n_vars * nodes[k] + i], R.phi[q][k]));
            F_qp[(long long)n_vars * t + i] = __dmul_rn(v, jxw);
        }
}

// One thread per (element, basis function, variable): the element's
// right-hand side entry summed over its quadrature points in order, added
// into the node's entry.  For simplices JxW(q) = (|det J| * w(q)) with one
// determinant; the product with phi is formed as phi * JxW either way.
template <int DIM, int TYPE>
__global__ void
fe_rhs_kernel(int n_elems, const int* elem_nodes, const double* X, const FeRule R, const double* U_qp, int n_vars,
              double* rhs)
{
    constexpr int NPE = fe_nodes(DIM, TYPE);
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n_elems * NPE * n_vars) return;
    const int i = (int)(t % n_vars);
    const int k = (int)((t / n_vars) % NPE);
    const int e = (int)(t / ((long long)n_vars * NPE));
    const int* nodes = elem_nodes + (long long)NPE * e;
    for (int j = 0; j < NPE; ++j)
        if (nodes[j] < 0) return;
    const double det = TYPE == IBX_FE_TENSOR_Q1 ? 0.0 : abs_det<DIM>(X, nodes);
    double acc = 0.0;
    for (int q = 0; q < R.n_qp; ++q)
    {
        const double jxw = TYPE == IBX_FE_TENSOR_Q1 ? elem_jxw<DIM, TYPE>(X, nodes, R, q) : __dmul_rn(det, R.w[q]);
        const double p_jxw = __dmul_rn(R.phi[q][k], jxw);
        acc = __dadd_rn(acc, __dmul_rn(U_qp[(long long)n_vars * ((long long)R.n_qp * e + q) + i], p_jxw));
    }
    atomicAdd(rhs + (long long)n_vars * nodes[k] + i, acc);
}

// The reference-cell corner of node k of a QUAD4 / HEX8 (libMesh's order):
// 0 for -1, 1 for +1 along each reference axis.
constexpr int Q1_CORNER[8][3] = { { 0, 0, 0 }, { 1, 0, 0 }, { 1, 1, 0 }, { 0, 1, 0 },
                                  { 0, 0, 1 }, { 1, 0, 1 }, { 1, 1, 1 }, { 0, 1, 1 } };

int
make_rule(const ibx_fe_mesh* mesh, const ibx_quad_rule* rule, FeRule& R)
{
    if (!mesh || !rule || (mesh->dim != 2 && mesh->dim != 3) || mesh->n_elems < 0 || mesh->n_nodes < 0)
        return IBX_E_ARG;
    if (mesh->elem_type != IBX_FE_SIMPLEX_P1 && mesh->elem_type != IBX_FE_TENSOR_Q1) return IBX_E_ARG;
    if (rule->n_points < 1 || rule->n_points > FE_MAX_QP || !rule->points || !rule->weights) return IBX_E_ARG;
    if (mesh->n_elems > 0 && (!mesh->elem_nodes || !mesh->X)) return IBX_E_ARG;
    const int dim = mesh->dim;
    R.n_qp = rule->n_points;
    for (int q = 0; q < R.n_qp; ++q)
    {
        for (int k = 0; k < FE_MAX_NODES; ++k)
        {
            R.phi[q][k] = 0.0;
            R.dphi[q][k][0] = R.dphi[q][k][1] = R.dphi[q][k][2] = 0.0;
        }
        const double* xi = rule->points + (long long)dim * q;
        if (mesh->elem_type == IBX_FE_SIMPLEX_P1)
        {
            double s = 0.0;
            for (int d = 0; d < dim; ++d)
            {
                R.phi[q][d + 1] = xi[d];
                s = s + xi[d];
            }
            R.phi[q][0] = 1.0 - s;
        }
        else
        {
            // phi_k = prod_c L_{corner}(xi_c), the product taken in axis order;
            // dphi_k/dxi_c the same product with L' = -1/2 or +1/2 on axis c
            for (int k = 0; k < (dim == 2 ? 4 : 8); ++k)
            {
                double L[3], dL[3];
                for (int c = 0; c < dim; ++c)
                {
                    L[c] = Q1_CORNER[k][c] ? 0.5 * (1.0 + xi[c]) : 0.5 * (1.0 - xi[c]);
                    dL[c] = Q1_CORNER[k][c] ? 0.5 : -0.5;
                }
                double p = L[0];
                for (int c = 1; c < dim; ++c) p = p * L[c];
                R.phi[q][k] = p;
                for (int c = 0; c < dim; ++c)
                {
                    double g = c == 0 ? dL[0] : L[0];
                    for (int a = 1; a < dim; ++a) g = g * (a == c ? dL[a] : L[a]);
                    R.dphi[q][k][c] = g;
                }
            }
        }
        R.w[q] = rule->weights[q];
    }
    return IBX_OK;
}
} // namespace
} // namespace ibx

extern "C" int
ibx_fe_quadrature_points(const ibx_fe_mesh* mesh, const ibx_quad_rule* rule, const double* F_nodes, int n_vars,
                         double* X_qp, double* F_JxW_qp, double* JxW, int* status, void* stream)
{
    using namespace ibx;
    FeRule R;
    const int rc = make_rule(mesh, rule, R);
    if (rc) return rc;
    if (F_nodes && (n_vars < 1 || !F_JxW_qp)) return IBX_E_ARG;
    if (!status) return IBX_E_ARG;
    const long long n = (long long)mesh->n_elems * R.n_qp;
    if (n == 0) return IBX_OK;
    if (n > 0x7fffffffLL) return IBX_E_TOO_LARGE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    const bool q1 = mesh->elem_type == IBX_FE_TENSOR_Q1;
#define IBX_FE_QP(DD, TT)                                                                                            \
    fe_qp_kernel<DD, TT><<<blocks, 256, 0, s>>>(mesh->n_elems, mesh->elem_nodes, mesh->X, R, F_nodes, n_vars, X_qp,  \
                                                F_JxW_qp, JxW, status)
    if (mesh->dim == 2)
    {
        if (q1)
            IBX_FE_QP(2, IBX_FE_TENSOR_Q1);
        else
            IBX_FE_QP(2, IBX_FE_SIMPLEX_P1);
    }
    else if (q1)
        IBX_FE_QP(3, IBX_FE_TENSOR_Q1);
    else
        IBX_FE_QP(3, IBX_FE_SIMPLEX_P1);
#undef IBX_FE_QP
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}

extern "C" int
ibx_fe_assemble_rhs(const ibx_fe_mesh* mesh, const ibx_quad_rule* rule, const double* U_qp, int n_vars, double* rhs,
                    void* stream)
{
    using namespace ibx;
    FeRule R;
    const int rc = make_rule(mesh, rule, R);
    if (rc) return rc;
    if (n_vars < 1 || !U_qp || !rhs) return IBX_E_ARG;
    const long long n = (long long)mesh->n_elems * fe_nodes(mesh->dim, mesh->elem_type) * n_vars;
    if (n == 0) return IBX_OK;
    if (n > 0x7fffffffLL) return IBX_E_TOO_LARGE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    const bool q1 = mesh->elem_type == IBX_FE_TENSOR_Q1;
#define IBX_FE_RHS(DD, TT)                                                                                           \
    fe_rhs_kernel<DD, TT><<<blocks, 256, 0, s>>>(mesh->n_elems, mesh->elem_nodes, mesh->X, R, U_qp, n_vars, rhs)
    if (mesh->dim == 2)
    {
        if (q1)
            IBX_FE_RHS(2, IBX_FE_TENSOR_Q1);
        else
            IBX_FE_RHS(2, IBX_FE_SIMPLEX_P1);
    }
    else if (q1)
        IBX_FE_RHS(3, IBX_FE_TENSOR_Q1);
    else
        IBX_FE_RHS(3, IBX_FE_SIMPLEX_P1);
#undef IBX_FE_RHS
    note_launches(1);
    return cudaGetLastError() == cudaSuccess ? IBX_OK : IBX_E_CUDA;
}
