// Post-processing of a face solution on the GPU: cell-unknown recovery, the k+1 reconstruction and
// its L2 error against a closed-form solution, element by element.
//
// Reference: Diffusion_HHO::HybridCoeffsBySolvingCellUnknowns (src/Discretizations/HHO/
// Diffusion_HHO.h:855-882: x_T = A_TT^{-1} (b_T - A_TF x_F) per element),
// ReconstructHigherOrderApproximationFromHybridCoeffs (:896-912: the reconstruction operator applied to
// [x_T; x_F]) and Diffusion_HHO::L2Error (:120-150: sqrt(sum_T |u_h - u|^2_T) / sqrt(sum_T |u|^2_T) by
// cell quadrature).
//
// Layout: per element its class, the unknown block of each local face (-1: Dirichlet), its centroid
// and A_TT^{-1} b_T; per class the dense local operators -A_TT^{-1} A_TF and the reconstruction, and
// at the cell quadrature points the weights, offsets from the centroid and reconstruction basis values.
// Elements of one class differ by a translation, so the class tables are shared (they stay in L1/L2);
// a caller without classes passes one class per element. One thread per element in FP64 (a one-off
// pass, bound by FP64 arithmetic and the sine evaluations, not by memory); the L2 sums go through
// per-CTA partials reduced in a fixed order, so the result is bitwise reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "fhg.h"

namespace {

constexpr int kPostThreads = 256;
constexpr int kPostMaxCtas = 152 * 8;
constexpr int kPostMaxCell = 20;       // cell basis functions (3D, k = 3)
constexpr int kPostMaxFaceDofs = 40;   // faces per element x face DOFs (3D, k = 3)
constexpr int kPostMaxRecon = 35;      // reconstruction basis functions (3D, degree 4)
constexpr int kPostMaxPoints = 512;

struct PostData {
    int dim, ne, nC, nFF, nF, nf, nR, nq;
    const int* cls;
    const int* faces;
    const double* centre;
    const double* cell_rhs;
    const double* sc;     // per class nC x nFF
    const double* rc;     // per class nR x (nC + nFF)
    const double* w;      // per class nq
    const double* off;    // per class nq x 3
    const double* basis;  // per class nq x nR
};

__device__ double block_sum_post(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sh[i];
    return t;  // valid in thread 0
}

// x_cells (optional) and, with exact = FHG_EXACT_SINE, per-CTA partial sums of |u_h - u|^2 and |u|^2.
__global__ void __launch_bounds__(kPostThreads) k_post(PostData D, const double* __restrict__ x, double* x_cells,
                                                       int exact, double* partials)
{
    __shared__ double sh[kPostThreads / 32];
    double err = 0.0, nrm = 0.0;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < D.ne; e += (long long)gridDim.x * blockDim.x) {
        const int c = D.cls[e];
        double hyb[kPostMaxCell + kPostMaxFaceDofs];
        for (int j = 0; j < D.nFF; j++) {
            const int g = D.faces[e * D.nF + j / D.nf];
            hyb[D.nC + j] = g >= 0 ? x[(long long)g * D.nf + j % D.nf] : 0.0;
        }
        const double* sc = D.sc + (long long)c * D.nC * D.nFF;
        for (int i = 0; i < D.nC; i++) {
            double v = D.cell_rhs[e * D.nC + i];
            for (int j = 0; j < D.nFF; j++) v += sc[i * D.nFF + j] * hyb[D.nC + j];
            hyb[i] = v;
            if (x_cells) x_cells[e * D.nC + i] = v;
        }
        if (exact != FHG_EXACT_SINE) continue;
        const int nh = D.nC + D.nFF;
        const double* rc = D.rc + (long long)c * D.nR * nh;
        double coef[kPostMaxRecon];
        for (int i = 0; i < D.nR; i++) {
            double s = 0.0;
            for (int j = 0; j < nh; j++) s += rc[i * nh + j] * hyb[j];
            coef[i] = s;
        }
        const double* w = D.w + (long long)c * D.nq;
        const double* off = D.off + (long long)c * D.nq * 3;
        const double* B = D.basis + (long long)c * D.nq * D.nR;
        for (int q = 0; q < D.nq; q++) {
            double uh = 0.0;
            for (int i = 0; i < D.nR; i++) uh += coef[i] * B[q * D.nR + i];
            double u = 1.0;
            for (int d = 0; d < D.dim; d++) u *= sinpi(D.centre[e * 3 + d] + off[q * 3 + d]);
            err += w[q] * (uh - u) * (uh - u);
            nrm += w[q] * u * u;
        }
    }
    if (exact != FHG_EXACT_SINE) return;
    const double te = block_sum_post(err, sh);
    const double tn = block_sum_post(nrm, sh);
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = te;
        partials[2 * blockIdx.x + 1] = tn;
    }
}

// Fixed-order sum of the partials (one thread: at most kPostMaxCtas pairs).
__global__ void k_post_finish(const double* partials, int n, double* out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double e = 0.0, u = 0.0;
    for (int i = 0; i < n; i++) {
        e += partials[2 * i];
        u += partials[2 * i + 1];
    }
    out[0] = e;
    out[1] = u;
}

}  // namespace

struct fhg_post {
    int device = 0;
    std::string err;
    PostData D{};
    std::vector<void*> allocs;
    double* partials = nullptr;
    double* sums = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

int post_fail(fhg_post* p, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (p) p->err = buf;
    return code;
}

#define PCK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return post_fail(p, FHG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int upload(fhg_post* p, const T* host, size_t n, const T** dev)
{
    void* d = nullptr;
    PCK(cudaMalloc(&d, sizeof(T) * std::max<size_t>(n, 1)));
    p->allocs.push_back(d);
    PCK(cudaMemcpy(d, host, sizeof(T) * n, cudaMemcpyHostToDevice));
    *dev = (const T*)d;
    return FHG_OK;
}

}  // namespace

extern "C" {

int fhg_post_create(fhg_post** out, int device, int dim, int n_elements, int n_classes, int n_cell, int n_face_dofs,
                    int n_recon, int n_points, const int* elem_class, const int* elem_faces, const double* elem_centre,
                    const double* cell_rhs, const double* solve_cells, const double* recon, const double* weights,
                    const double* offsets, const double* basis)
{
    if (!out) return FHG_ERR_INVALID_ARG;
    fhg_post* p = new fhg_post();
    *out = p;
    p->device = device;
    if (dim != 2 && dim != 3) return post_fail(p, FHG_ERR_INVALID_ARG, "dimension %d", dim);
    if (n_elements <= 0 || n_classes <= 0 || n_cell <= 0 || n_recon <= 0 || n_points <= 0 ||
        n_face_dofs <= 0 || n_face_dofs % (dim + 1) != 0)
        return post_fail(p, FHG_ERR_INVALID_ARG, "bad table sizes");
    if (n_cell > kPostMaxCell || n_face_dofs > kPostMaxFaceDofs || n_recon > kPostMaxRecon || n_points > kPostMaxPoints)
        return post_fail(p, FHG_ERR_UNSUPPORTED, "element tables larger than supported (%d cell, %d face, %d recon, %d points)",
                         n_cell, n_face_dofs, n_recon, n_points);
    if (!elem_class || !elem_faces || !elem_centre || !cell_rhs || !solve_cells || !recon || !weights || !offsets || !basis)
        return post_fail(p, FHG_ERR_INVALID_ARG, "null table");
    for (int e = 0; e < n_elements; e++)
        if (elem_class[e] < 0 || elem_class[e] >= n_classes)
            return post_fail(p, FHG_ERR_INVALID_ARG, "element %d: class %d out of range", e, elem_class[e]);
    PCK(cudaSetDevice(device));
    PostData& D = p->D;
    D.dim = dim;
    D.ne = n_elements;
    D.nC = n_cell;
    D.nFF = n_face_dofs;
    D.nF = dim + 1;
    D.nf = n_face_dofs / (dim + 1);
    D.nR = n_recon;
    D.nq = n_points;
    const size_t ne = n_elements, nc = n_classes;
    int rc;
    if ((rc = upload(p, elem_class, ne, &D.cls)) || (rc = upload(p, elem_faces, ne * D.nF, &D.faces)) ||
        (rc = upload(p, elem_centre, ne * 3, &D.centre)) || (rc = upload(p, cell_rhs, ne * n_cell, &D.cell_rhs)) ||
        (rc = upload(p, solve_cells, nc * n_cell * n_face_dofs, &D.sc)) ||
        (rc = upload(p, recon, nc * n_recon * (n_cell + n_face_dofs), &D.rc)) ||
        (rc = upload(p, weights, nc * n_points, &D.w)) || (rc = upload(p, offsets, nc * n_points * 3, &D.off)) ||
        (rc = upload(p, basis, nc * n_points * n_recon, &D.basis)))
        return rc;
    void* d = nullptr;
    PCK(cudaMalloc(&d, sizeof(double) * (2 * kPostMaxCtas + 2)));
    p->allocs.push_back(d);
    p->partials = (double*)d;
    p->sums = p->partials + 2 * kPostMaxCtas;
    PCK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    PCK(cudaEventCreate(&p->ev0));
    PCK(cudaEventCreate(&p->ev1));
    return FHG_OK;
}

int fhg_post_run(fhg_post* p, const double* x_faces, double* x_cells, int exact, double* rel_l2_error, double* elapsed_ms)
{
    if (!p || !p->stream) return FHG_ERR_INVALID_ARG;
    if (!x_faces) return post_fail(p, FHG_ERR_INVALID_ARG, "null face solution");
    if (exact != FHG_EXACT_NONE && exact != FHG_EXACT_SINE) return post_fail(p, FHG_ERR_INVALID_ARG, "unknown exact solution %d", exact);
    if (exact == FHG_EXACT_SINE && !rel_l2_error) return post_fail(p, FHG_ERR_INVALID_ARG, "null error output");
    PCK(cudaSetDevice(p->device));
    const int grid = (int)std::min<long long>(kPostMaxCtas, ((long long)p->D.ne + kPostThreads - 1) / kPostThreads);
    PCK(cudaEventRecord(p->ev0, p->stream));
    k_post<<<grid, kPostThreads, 0, p->stream>>>(p->D, x_faces, x_cells, exact, p->partials);
    PCK(cudaGetLastError());
    if (exact == FHG_EXACT_SINE) {
        k_post_finish<<<1, 32, 0, p->stream>>>(p->partials, grid, p->sums);
        PCK(cudaGetLastError());
    }
    PCK(cudaEventRecord(p->ev1, p->stream));
    double s[2] = {0.0, 0.0};
    if (exact == FHG_EXACT_SINE) PCK(cudaMemcpyAsync(s, p->sums, sizeof(s), cudaMemcpyDeviceToHost, p->stream));
    PCK(cudaStreamSynchronize(p->stream));
    if (exact == FHG_EXACT_SINE) *rel_l2_error = s[1] > 0 ? std::sqrt(s[0]) / std::sqrt(s[1]) : std::sqrt(s[0]);
    if (elapsed_ms) {
        float ms = 0.f;
        PCK(cudaEventElapsedTime(&ms, p->ev0, p->ev1));
        *elapsed_ms = ms;
    }
    return FHG_OK;
}

const char* fhg_post_last_error(const fhg_post* p) { return p ? p->err.c_str() : "null post-processing handle"; }

void fhg_post_destroy(fhg_post* p)
{
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (void* d : p->allocs) cudaFree(d);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

}  // extern "C"
