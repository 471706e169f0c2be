// k_diag.cu -- microstructure diagnostics on row-major FP64 fields (the
// handle's gathered state), all deterministic (integer atomics or fixed-order
// FP64 partials):
//  * level-set interface: area, edge-count perimeter and bounding box of
//    {f >= level} (Kobayashi dendrite extent and tip positions);
//  * grains: connected components (4-neighbour, through periodic wraps) of
//    cells labelled by the dominant order parameter argmax_k eta_k where
//    max_k eta_k >= threshold -- grain count, labelled cells, mean area;
//  * grain-boundary length between every pair of labels (grain growth:
//    boundary network; sintering: neck widths, with cells labelled only where
//    the concentration c >= level).
// No reference counterpart: the reference's analysis scripts compare fields
// only (mean absolute error, graingrowth/end2enderror.py:34, which
// amps_compare_all also reports).
#include "amps_internal.cuh"
#include "amps_kernels.h"

#include <algorithm>

namespace amps {

namespace {

constexpr int kDT = 256;

__device__ __forceinline__ int wrap_or_out(int i, int n, int bc)
{
    if (i >= 0 && i < n) return i;
    if (bc == 0) return i < 0 ? i + n : i - n;
    return -1;  // zero-flux: no neighbour outside the domain
}

__global__ void interface_kernel(const double *f, int nx, int ny, int bc, double level, unsigned long long *acc,
                                 int *box)
{
    const int64_t n = (int64_t)nx * ny;
    unsigned long long in = 0, ex = 0, ey = 0;
    for (int64_t i = blockIdx.x * (int64_t)kDT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kDT) {
        const int x = (int)(i % nx), y = (int)(i / nx);
        const bool a = f[i] >= level;
        if (a) {
            ++in;
            atomicMin(&box[0], x);
            atomicMax(&box[1], x);
            atomicMin(&box[2], y);
            atomicMax(&box[3], y);
        }
        const int xr = wrap_or_out(x + 1, nx, bc), yd = wrap_or_out(y + 1, ny, bc);
        if (xr >= 0 && a != (f[(int64_t)y * nx + xr] >= level)) ++ex;
        if (yd >= 0 && a != (f[(int64_t)yd * nx + x] >= level)) ++ey;
    }
    for (int o = 16; o > 0; o >>= 1) {
        in += __shfl_xor_sync(0xffffffffu, in, o);
        ex += __shfl_xor_sync(0xffffffffu, ex, o);
        ey += __shfl_xor_sync(0xffffffffu, ey, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], in);
        atomicAdd(&acc[1], ex);
        atomicAdd(&acc[2], ey);
    }
}

// label = argmax_k eta_k (fields e0 .. e0+q-1) where max >= thr and, when
// conc is given, conc >= clevel; else -1.  Ties go to the lower index.
__global__ void label_kernel(const double *fields, int e0, int q, int64_t n, double thr, const double *conc,
                             double clevel, int *lab, int *parent)
{
    for (int64_t i = blockIdx.x * (int64_t)kDT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kDT) {
        int best = -1;
        double bv = 0.0;
        for (int k = 0; k < q; ++k) {
            const double v = fields[(int64_t)(e0 + k) * n + i];
            if (best < 0 || v > bv) {
                best = k;
                bv = v;
            }
        }
        int l = (bv >= thr) ? best : -1;
        if (conc && !(conc[i] >= clevel)) l = -1;
        lab[i] = l;
        if (parent) parent[i] = l >= 0 ? (int)i : -1;
    }
}

// A non-root always points to a smaller index (links go from the larger root
// to the smaller), so a walk from i ends within i steps; the cap (cells + 1)
// only guards against a corrupted array and raises flag bit 2.
__device__ __forceinline__ int find_root(const int *parent, int i, int64_t cap, int *flags)
{
    for (int64_t it = 0; it < cap; ++it) {
        const int p = ((volatile const int *)parent)[i];
        if (p == i) return i;
        i = p;
    }
    atomicOr(flags, 4);
    return i;
}

// Each retry continues from a strictly smaller index, so this ends within
// `cap` rounds as well.
__device__ __forceinline__ void unite(int *parent, int a, int b, int64_t cap, int *flags)
{
    for (int64_t it = 0; it < cap; ++it) {
        a = find_root(parent, a, cap, flags);
        b = find_root(parent, b, cap, flags);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicMin(&parent[a], b);  // link the larger root under the smaller
        if (old == a) return;
        a = old;  // a was re-linked meanwhile: continue from its new parent
    }
    atomicOr(flags, 4);
}

__global__ void union_kernel(const int *lab, int *parent, int nx, int ny, int bc, int *flags)
{
    const int64_t n = (int64_t)nx * ny;
    for (int64_t i = blockIdx.x * (int64_t)kDT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kDT) {
        const int l = lab[i];
        if (l < 0) continue;
        const int x = (int)(i % nx), y = (int)(i / nx);
        const int xr = wrap_or_out(x + 1, nx, bc), yd = wrap_or_out(y + 1, ny, bc);
        if (xr >= 0) {
            const int64_t j = (int64_t)y * nx + xr;
            if (lab[j] == l) unite(parent, (int)i, (int)j, n + 1, flags);
        }
        if (yd >= 0) {
            const int64_t j = (int64_t)yd * nx + x;
            if (lab[j] == l) unite(parent, (int)i, (int)j, n + 1, flags);
        }
    }
}

__global__ void count_roots_kernel(const int *lab, const int *parent, int64_t n, unsigned long long *acc)
{
    unsigned long long roots = 0, cells = 0;
    for (int64_t i = blockIdx.x * (int64_t)kDT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kDT) {
        if (lab[i] < 0) continue;
        ++cells;
        roots += parent[i] == (int)i;
    }
    for (int o = 16; o > 0; o >>= 1) {
        roots += __shfl_xor_sync(0xffffffffu, roots, o);
        cells += __shfl_xor_sync(0xffffffffu, cells, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], roots);
        atomicAdd(&acc[1], cells);
    }
}

// Boundary edges between differently labelled neighbours, per unordered
// label pair: acc[(a*q + b)*2 + 0] x-edges (length dy each), [.. + 1] y-edges.
__global__ void boundary_kernel(const int *lab, int nx, int ny, int bc, int q, unsigned long long *acc)
{
    const int64_t n = (int64_t)nx * ny;
    for (int64_t i = blockIdx.x * (int64_t)kDT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kDT) {
        const int l = lab[i];
        if (l < 0) continue;
        const int x = (int)(i % nx), y = (int)(i / nx);
        const int xr = wrap_or_out(x + 1, nx, bc), yd = wrap_or_out(y + 1, ny, bc);
        if (xr >= 0) {
            const int m = lab[(int64_t)y * nx + xr];
            if (m >= 0 && m != l) atomicAdd(&acc[((int64_t)min(l, m) * q + max(l, m)) * 2], 1ull);
        }
        if (yd >= 0) {
            const int m = lab[(int64_t)yd * nx + x];
            if (m >= 0 && m != l) atomicAdd(&acc[((int64_t)min(l, m) * q + max(l, m)) * 2 + 1], 1ull);
        }
    }
}

__global__ void box_init_kernel(int *box)
{
    if (threadIdx.x < 4) box[threadIdx.x] = (threadIdx.x & 1) ? -1 : 0x7fffffff;
}

// max |a-b|, sum (a-b)^2, sum |a-b| per block (fixed order within the block)
__global__ void compare3_kernel(const double *a, const double *b, int64_t n, double *partials)
{
    __shared__ double red[3][kDT / 32];
    double mx = 0.0, ss = 0.0, sa = 0.0;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    for (int64_t i = lo + threadIdx.x; i < hi; i += kDT) {
        const double d = a[i] - b[i];
        mx = (fabs(d) > mx || !(d == d)) ? fabs(d) : mx;
        ss += d * d;
        sa += fabs(d);
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double m2 = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = (m2 > mx || !(m2 == m2)) ? m2 : mx;
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        sa += __shfl_xor_sync(0xffffffffu, sa, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = mx;
        red[1][threadIdx.x >> 5] = ss;
        red[2][threadIdx.x >> 5] = sa;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0, s2 = 0.0, s1 = 0.0;
        for (int w = 0; w < kDT / 32; ++w) {
            m = (red[0][w] > m || !(red[0][w] == red[0][w])) ? red[0][w] : m;
            s2 += red[1][w];
            s1 += red[2][w];
        }
        partials[3 * blockIdx.x] = m;
        partials[3 * blockIdx.x + 1] = s2;
        partials[3 * blockIdx.x + 2] = s1;
    }
}

__global__ void compare3_final_kernel(const double *partials, int np, int64_t n, double *out)
{
    if (threadIdx.x != 0) return;
    double m = 0.0, s2 = 0.0, s1 = 0.0;
    for (int k = 0; k < np; ++k) {
        const double v = partials[3 * k];
        m = (v > m || !(v == v)) ? v : m;
        s2 += partials[3 * k + 1];
        s1 += partials[3 * k + 2];
    }
    out[0] = m;
    out[1] = sqrt(s2 / (double)n);
    out[2] = s1 / (double)n;
}

int grid_for_diag(int64_t n) { return (int)std::min<int64_t>((n + kDT - 1) / kDT, 152 * 8); }

}  // namespace

cudaError_t diag_interface(const double *f, int nx, int ny, int bc, double level, unsigned long long *acc, int *box,
                           cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(acc, 0, 3 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    box_init_kernel<<<1, 32, 0, s>>>(box);
    interface_kernel<<<grid_for_diag((int64_t)nx * ny), kDT, 0, s>>>(f, nx, ny, bc, level, acc, box);
    return cudaGetLastError();
}

cudaError_t diag_grains(const double *fields, int e0, int q, int nx, int ny, int bc, double thr, const double *conc,
                        double clevel, int *lab, int *parent, unsigned long long *acc, int *flags, cudaStream_t s)
{
    const int64_t n = (int64_t)nx * ny;
    const int g = grid_for_diag(n);
    cudaError_t e = cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    label_kernel<<<g, kDT, 0, s>>>(fields, e0, q, n, thr, conc, clevel, lab, parent);
    union_kernel<<<g, kDT, 0, s>>>(lab, parent, nx, ny, bc, flags);
    count_roots_kernel<<<g, kDT, 0, s>>>(lab, parent, n, acc);
    return cudaGetLastError();
}

cudaError_t diag_boundaries(const double *fields, int e0, int q, int nx, int ny, int bc, const double *conc,
                            double clevel, int *lab, unsigned long long *acc, cudaStream_t s)
{
    const int64_t n = (int64_t)nx * ny;
    const int g = grid_for_diag(n);
    cudaError_t e = cudaMemsetAsync(acc, 0, (size_t)q * q * 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    label_kernel<<<g, kDT, 0, s>>>(fields, e0, q, n, -1e300, conc, clevel, lab, nullptr);
    boundary_kernel<<<g, kDT, 0, s>>>(lab, nx, ny, bc, q, acc);
    return cudaGetLastError();
}

cudaError_t diag_compare3(const double *a, const double *b, int64_t n, double *partials, int np, double *out,
                          cudaStream_t s)
{
    compare3_kernel<<<np, kDT, 0, s>>>(a, b, n, partials);
    compare3_final_kernel<<<1, 32, 0, s>>>(partials, np, n, out);
    return cudaGetLastError();
}

}  // namespace amps
