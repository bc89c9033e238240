// Static condensation and assembly of the finest face system on the GPU.
//
// Reference: Diffusion_HHO::Assemble's condensation (src/Discretizations/HHO/Diffusion_HHO.h:627-638):
// with the cell unknowns of every element eliminated, the face operator is
//   A = A_FF - A_TF^T A_TT^{-1} A_TF,   b = b_F - A_TF^T A_TT^{-1} b_T,
// assembled element by element over the interior faces.
//
// Input: per class (elements that differ by a translation share their local operator; a caller
// without classes passes one class per element) the local operator before condensation, cells
// first; per element its class, its faces' unknown blocks (-1: Dirichlet) and b_T; per unknown face
// block its two elements with the face's local index in each. Steps, all in FP64:
//   1. per class: A_TT^{-1} by Gauss-Jordan elimination with partial pivoting; the Schur complement
//      S = A_FF - A_TF^T (A_TT^{-1} A_TF) and the source map G = -A_TF^T A_TT^{-1}
//      (n_face_dofs x n_cell) are kept;
//   2. per face block row: the sorted union of the unknown faces of its two elements is the row's
//      block columns (counted, then offsets by a three-pass scan);
//   3. per face block row: the values, S of the first element then of the second added into the
//      row's positions in that order, and b_I = sum over the two elements of G b_T, restricted to
//      the face's rows (the same order as the host assembly, so off-diagonal blocks are copies and
//      diagonal blocks one addition).
// Every row is written by one thread: no atomics, the result is bitwise reproducible. The output is
// the scalar CSR the solve phase takes (fhg_set_level): rows I * nf + a, columns J * nf + c.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "fhg.h"

namespace {

constexpr int kCondThreads = 256;
constexpr int kCondMaxCell = 20;      // cell unknowns (3D, k = 3)
constexpr int kCondMaxFaceDofs = 40;  // faces per element x face DOFs (3D, k = 3)
constexpr int kCondMaxRowBlocks = 8;  // block columns of a face row: 2 (dim + 1) - 1 <= 7

struct CondData {
    int dim, ne, ncls, nC, nFF, nF, nf, nI;
    const int* cls;
    const int* elem_faces;
    const int* face_elems;
    const double* local;   // per class nH x nH
    const double* b_cell;  // per element nC
    double* S;             // per class nFF x nFF
    double* G;             // per class nFF x nC
    int* status;           // 1: a singular A_TT
};

// Step 1, one thread per class: Gauss-Jordan elimination with partial pivoting of [A_TT | I] gives
// A_TT^{-1}; then S = A_FF - A_TF^T (A_TT^{-1} A_TF) and G = -A_TF^T A_TT^{-1}. NC = cell unknowns.
template <int NC>
__global__ void __launch_bounds__(64) k_condense_classes(CondData D)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= D.ncls) return;
    const int nFF = D.nFF, nH = NC + nFF;
    const double* A = D.local + (long long)c * nH * nH;
    double M[NC][NC], V[NC][NC];
    for (int i = 0; i < NC; i++)
        for (int j = 0; j < NC; j++) {
            M[i][j] = A[i * nH + j];
            V[i][j] = i == j ? 1.0 : 0.0;
        }
    for (int k = 0; k < NC; k++) {
        int piv = k;
        for (int i = k + 1; i < NC; i++)
            if (fabs(M[i][k]) > fabs(M[piv][k])) piv = i;
        if (M[piv][k] == 0.0) {
            atomicExch(D.status, 1);
            return;
        }
        if (piv != k)
            for (int j = 0; j < NC; j++) {
                double t = M[k][j]; M[k][j] = M[piv][j]; M[piv][j] = t;
                t = V[k][j]; V[k][j] = V[piv][j]; V[piv][j] = t;
            }
        const double inv = 1.0 / M[k][k];
        for (int j = 0; j < NC; j++) { M[k][j] *= inv; V[k][j] *= inv; }
        for (int i = 0; i < NC; i++) {
            if (i == k) continue;
            const double f = M[i][k];
            if (f == 0.0) continue;
            for (int j = 0; j < NC; j++) { M[i][j] -= f * M[k][j]; V[i][j] -= f * V[k][j]; }
        }
    }
    // V = A_TT^{-1}; X(:, j) = V A_TF(:, j) formed column by column
    double* S = D.S + (long long)c * nFF * nFF;
    double* G = D.G + (long long)c * nFF * NC;
    for (int j = 0; j < nFF; j++) {
        double x[NC];
        for (int t = 0; t < NC; t++) {
            double v = 0.0;
            for (int u = 0; u < NC; u++) v += V[t][u] * A[u * nH + NC + j];
            x[t] = v;
        }
        for (int i = 0; i < nFF; i++) {
            double s = A[(NC + i) * nH + NC + j];
            for (int t = 0; t < NC; t++) s -= A[t * nH + NC + i] * x[t];
            S[i * nFF + j] = s;
        }
    }
    for (int i = 0; i < nFF; i++)
        for (int j = 0; j < NC; j++) {
            double v = 0.0;
            for (int t = 0; t < NC; t++) v += A[t * nH + NC + i] * V[t][j];
            G[i * NC + j] = -v;
        }
}

// The sorted block columns of face row I (the unknown faces of its two elements).
__device__ int row_columns(const CondData& D, int I, int* cols)
{
    int n = 0;
    for (int side = 0; side < 2; side++) {
        const int e = D.face_elems[(long long)I * 4 + 2 * side];
        if (e < 0) continue;
        for (int lf = 0; lf < D.nF; lf++) {
            const int g = D.elem_faces[(long long)e * D.nF + lf];
            if (g < 0) continue;
            bool seen = false;
            for (int q = 0; q < n; q++) seen |= cols[q] == g;
            if (!seen && n < kCondMaxRowBlocks) cols[n++] = g;
        }
    }
    for (int i = 1; i < n; i++) {   // insertion sort (n <= 7)
        const int v = cols[i];
        int j = i - 1;
        while (j >= 0 && cols[j] > v) { cols[j + 1] = cols[j]; j--; }
        cols[j + 1] = v;
    }
    return n;
}

// Step 2: block columns per face row.
__global__ void __launch_bounds__(kCondThreads) k_count(CondData D, int* counts)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= D.nI) return;
    int cols[kCondMaxRowBlocks];
    counts[I] = row_columns(D, I, cols);
}

// Three-pass exclusive scan: per-CTA totals, a scan of the totals by one CTA, per-CTA scans with
// the offsets added. out[n] = total.
__global__ void __launch_bounds__(kCondThreads) k_scan_totals(const int* in, int n, long long* totals)
{
    __shared__ long long sh[kCondThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    sh[threadIdx.x] = i < n ? in[i] : 0;
    __syncthreads();
    for (int o = kCondThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = sh[0];
}

__global__ void k_scan_offsets(long long* totals, int nblocks)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long run = 0;
    for (int b = 0; b < nblocks; b++) {
        const long long t = totals[b];
        totals[b] = run;
        run += t;
    }
    totals[nblocks] = run;
}

__global__ void __launch_bounds__(kCondThreads) k_scan_apply(const int* in, int n, const long long* offsets, long long* out)
{
    __shared__ long long sh[kCondThreads];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const long long v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kCondThreads; o <<= 1) {   // inclusive Hillis-Steele scan
        const long long t = (int)threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = offsets[blockIdx.x] + sh[threadIdx.x] - v;
    if (i == n - 1) out[n] = offsets[blockIdx.x] + sh[threadIdx.x];
}

// Step 3: row I's scalar rows, column indices, values and right-hand side.
__global__ void __launch_bounds__(kCondThreads) k_fill(CondData D, const long long* block_start, int* rowptr,
                                                       int* colidx, double* vals, double* b)
{
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= D.nI) return;
    const int nf = D.nf, nC = D.nC, nFF = D.nFF;
    int cols[kCondMaxRowBlocks];
    const int nb = row_columns(D, I, cols);
    const long long base = block_start[I] * nf * nf;   // first scalar entry of the block row
    const int width = nb * nf;                         // scalar entries per row
    for (int a = 0; a < nf; a++) {
        const long long r0 = base + (long long)a * width;
        rowptr[(long long)I * nf + a] = (int)r0;
        for (int q = 0; q < nb; q++)
            for (int cc = 0; cc < nf; cc++) {
                colidx[r0 + q * nf + cc] = cols[q] * nf + cc;
                vals[r0 + q * nf + cc] = 0.0;
            }
    }
    if (I == D.nI - 1) rowptr[(long long)D.nI * nf] = (int)(base + (long long)nf * width);
    double bI[kCondMaxFaceDofs];
    for (int a = 0; a < nf; a++) bI[a] = 0.0;
    for (int side = 0; side < 2; side++) {
        const int e = D.face_elems[(long long)I * 4 + 2 * side];
        const int lfi = D.face_elems[(long long)I * 4 + 2 * side + 1];
        if (e < 0 || lfi < 0) continue;
        const int c = D.cls[e];
        const double* S = D.S + (long long)c * nFF * nFF;
        const double* G = D.G + (long long)c * nFF * nC;
        for (int lf = 0; lf < D.nF; lf++) {
            const int g = D.elem_faces[(long long)e * D.nF + lf];
            if (g < 0) continue;
            int q = 0;
            while (q < nb && cols[q] != g) q++;
            for (int a = 0; a < nf; a++) {
                double* dst = vals + base + (long long)a * width + q * nf;
                for (int cc = 0; cc < nf; cc++) dst[cc] += S[(lfi * nf + a) * nFF + lf * nf + cc];
            }
        }
        const double* bT = D.b_cell + (long long)e * nC;
        for (int a = 0; a < nf; a++) {
            double s = 0.0;
            for (int t = 0; t < nC; t++) s += G[(lfi * nf + a) * nC + t] * bT[t];
            bI[a] += s;
        }
    }
    for (int a = 0; a < nf; a++) b[(long long)I * nf + a] = bI[a];
}

}  // namespace

struct fhg_cond {
    int device = 0;
    std::string err;
    CondData D{};
    std::vector<void*> allocs;
    int* counts = nullptr;
    long long* block_start = nullptr;
    long long* totals = nullptr;
    int* rowptr = nullptr;
    int* colidx = nullptr;
    double* vals = nullptr;
    double* b = nullptr;
    long long nnz = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

int cond_fail(fhg_cond* p, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (p) p->err = buf;
    return code;
}

#define DCK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return cond_fail(p, FHG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dev_alloc(fhg_cond* p, T** out, size_t n)
{
    void* d = nullptr;
    DCK(cudaMalloc(&d, sizeof(T) * std::max<size_t>(n, 1)));
    p->allocs.push_back(d);
    *out = (T*)d;
    return FHG_OK;
}

template <class T>
int dev_upload(fhg_cond* p, const T* host, size_t n, const T** out)
{
    T* d = nullptr;
    int rc = dev_alloc(p, &d, n);
    if (rc) return rc;
    DCK(cudaMemcpy(d, host, sizeof(T) * n, cudaMemcpyHostToDevice));
    *out = d;
    return FHG_OK;
}

}  // namespace

extern "C" {

int fhg_cond_create(fhg_cond** out, int device, int dim, int n_elements, int n_classes, int n_cell, int n_face_dofs,
                    int n_face_blocks, const int* elem_class, const int* elem_faces, const int* face_elems,
                    const double* local, const double* b_cell)
{
    if (!out) return FHG_ERR_INVALID_ARG;
    fhg_cond* p = new fhg_cond();
    *out = p;
    p->device = device;
    if (dim != 2 && dim != 3) return cond_fail(p, FHG_ERR_INVALID_ARG, "dimension %d", dim);
    if (n_elements <= 0 || n_classes <= 0 || n_cell <= 0 || n_face_blocks <= 0 || n_face_dofs <= 0 ||
        n_face_dofs % (dim + 1) != 0)
        return cond_fail(p, FHG_ERR_INVALID_ARG, "bad table sizes");
    if (n_cell > kCondMaxCell || n_face_dofs > kCondMaxFaceDofs ||
        (n_cell != 3 && n_cell != 4 && n_cell != 6 && n_cell != 10 && n_cell != 20))
        return cond_fail(p, FHG_ERR_UNSUPPORTED, "element larger than supported (%d cell, %d face unknowns)", n_cell,
                         n_face_dofs);
    if (!elem_class || !elem_faces || !face_elems || !local || !b_cell) return cond_fail(p, FHG_ERR_INVALID_ARG, "null table");
    const int nF = dim + 1;
    for (int e = 0; e < n_elements; e++) {
        if (elem_class[e] < 0 || elem_class[e] >= n_classes)
            return cond_fail(p, FHG_ERR_INVALID_ARG, "element %d: class %d out of range", e, elem_class[e]);
        for (int lf = 0; lf < nF; lf++)
            if (elem_faces[(size_t)e * nF + lf] >= n_face_blocks)
                return cond_fail(p, FHG_ERR_INVALID_ARG, "element %d: face block out of range", e);
    }
    for (int I = 0; I < n_face_blocks; I++)
        for (int side = 0; side < 2; side++) {
            const int e = face_elems[(size_t)I * 4 + 2 * side], lf = face_elems[(size_t)I * 4 + 2 * side + 1];
            if (e >= n_elements || (e >= 0 && (lf < 0 || lf >= nF || elem_faces[(size_t)e * nF + lf] != I)))
                return cond_fail(p, FHG_ERR_INVALID_ARG, "face block %d: element %d / local face %d inconsistent", I, e, lf);
        }
    DCK(cudaSetDevice(device));
    CondData& D = p->D;
    D.dim = dim;
    D.ne = n_elements;
    D.ncls = n_classes;
    D.nC = n_cell;
    D.nFF = n_face_dofs;
    D.nF = nF;
    D.nf = n_face_dofs / nF;
    D.nI = n_face_blocks;
    const size_t ne = n_elements, nc = n_classes, nH = n_cell + n_face_dofs;
    int rc;
    if ((rc = dev_upload(p, elem_class, ne, &D.cls)) || (rc = dev_upload(p, elem_faces, ne * nF, &D.elem_faces)) ||
        (rc = dev_upload(p, face_elems, (size_t)n_face_blocks * 4, &D.face_elems)) ||
        (rc = dev_upload(p, local, nc * nH * nH, &D.local)) || (rc = dev_upload(p, b_cell, ne * n_cell, &D.b_cell)) ||
        (rc = dev_alloc(p, &D.S, nc * n_face_dofs * n_face_dofs)) || (rc = dev_alloc(p, &D.G, nc * n_face_dofs * n_cell)) ||
        (rc = dev_alloc(p, &D.status, 1)) || (rc = dev_alloc(p, &p->counts, (size_t)n_face_blocks)) ||
        (rc = dev_alloc(p, &p->block_start, (size_t)n_face_blocks + 1)) ||
        (rc = dev_alloc(p, &p->totals, (size_t)(n_face_blocks + kCondThreads - 1) / kCondThreads + 1)) ||
        (rc = dev_alloc(p, &p->b, (size_t)n_face_blocks * D.nf)) ||
        (rc = dev_alloc(p, &p->rowptr, (size_t)n_face_blocks * D.nf + 1)))
        return rc;
    DCK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    DCK(cudaEventCreate(&p->ev0));
    DCK(cudaEventCreate(&p->ev1));
    return FHG_OK;
}

int fhg_cond_run(fhg_cond* p, long long* nnz, double* elapsed_ms)
{
    if (!p || !p->stream) return FHG_ERR_INVALID_ARG;
    DCK(cudaSetDevice(p->device));
    CondData& D = p->D;
    const int nI = D.nI, nf = D.nf;
    const int grid = (nI + kCondThreads - 1) / kCondThreads;
    cudaStream_t s = p->stream;
    DCK(cudaMemsetAsync(D.status, 0, sizeof(int), s));
    DCK(cudaEventRecord(p->ev0, s));
    const int cgrid = (D.ncls + 63) / 64;
    switch (D.nC) {
    case 3: k_condense_classes<3><<<cgrid, 64, 0, s>>>(D); break;
    case 4: k_condense_classes<4><<<cgrid, 64, 0, s>>>(D); break;
    case 6: k_condense_classes<6><<<cgrid, 64, 0, s>>>(D); break;
    case 10: k_condense_classes<10><<<cgrid, 64, 0, s>>>(D); break;
    case 20: k_condense_classes<20><<<cgrid, 64, 0, s>>>(D); break;
    default: return cond_fail(p, FHG_ERR_UNSUPPORTED, "%d cell unknowns per element", D.nC);
    }
    k_count<<<grid, kCondThreads, 0, s>>>(D, p->counts);
    k_scan_totals<<<grid, kCondThreads, 0, s>>>(p->counts, nI, p->totals);
    k_scan_offsets<<<1, 32, 0, s>>>(p->totals, grid);
    k_scan_apply<<<grid, kCondThreads, 0, s>>>(p->counts, nI, p->totals, p->block_start);
    DCK(cudaGetLastError());
    long long blocks = 0;
    int status = 0;
    DCK(cudaMemcpyAsync(&blocks, p->block_start + nI, sizeof(long long), cudaMemcpyDeviceToHost, s));
    DCK(cudaMemcpyAsync(&status, D.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    DCK(cudaStreamSynchronize(s));
    if (status) return cond_fail(p, FHG_ERR_SINGULAR_BLOCK, "singular cell block in a local operator");
    const long long n_scalar = blocks * nf * nf;
    if (n_scalar > 0x7fffffffLL) return cond_fail(p, FHG_ERR_TOO_LARGE, "%lld entries exceed 32-bit indices", n_scalar);
    if (n_scalar != p->nnz) {
        for (void* d : {(void*)p->colidx, (void*)p->vals})
            if (d) {
                cudaFree(d);
                p->allocs.erase(std::find(p->allocs.begin(), p->allocs.end(), d));
            }
        p->colidx = nullptr;
        p->vals = nullptr;
        int rc;
        if ((rc = dev_alloc(p, &p->colidx, (size_t)n_scalar)) || (rc = dev_alloc(p, &p->vals, (size_t)n_scalar))) return rc;
        p->nnz = n_scalar;
    }
    k_fill<<<grid, kCondThreads, 0, s>>>(D, p->block_start, p->rowptr, p->colidx, p->vals, p->b);
    DCK(cudaGetLastError());
    DCK(cudaEventRecord(p->ev1, s));
    DCK(cudaStreamSynchronize(s));
    if (nnz) *nnz = n_scalar;
    if (elapsed_ms) {
        float ms = 0.f;
        DCK(cudaEventElapsedTime(&ms, p->ev0, p->ev1));
        *elapsed_ms = ms;
    }
    return FHG_OK;
}

int fhg_cond_result(fhg_cond* p, int** rowptr, int** colidx, double** vals, double** b)
{
    if (!p || p->nnz < 0) return FHG_ERR_NOT_READY;
    if (rowptr) *rowptr = p->rowptr;
    if (colidx) *colidx = p->colidx;
    if (vals) *vals = p->vals;
    if (b) *b = p->b;
    return FHG_OK;
}

int fhg_cond_download(fhg_cond* p, int* rowptr, int* colidx, double* vals, double* b)
{
    if (!p || p->nnz < 0) return FHG_ERR_NOT_READY;
    DCK(cudaSetDevice(p->device));
    const size_t n = (size_t)p->D.nI * p->D.nf;
    if (rowptr) DCK(cudaMemcpy(rowptr, p->rowptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    if (colidx) DCK(cudaMemcpy(colidx, p->colidx, sizeof(int) * (size_t)p->nnz, cudaMemcpyDeviceToHost));
    if (vals) DCK(cudaMemcpy(vals, p->vals, sizeof(double) * (size_t)p->nnz, cudaMemcpyDeviceToHost));
    if (b) DCK(cudaMemcpy(b, p->b, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return FHG_OK;
}

const char* fhg_cond_last_error(const fhg_cond* p) { return p ? p->err.c_str() : "null condensation handle"; }

void fhg_cond_destroy(fhg_cond* p)
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
