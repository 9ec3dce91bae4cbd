// (T) triples correction of a converged closed-shell CCSD: the energy kernels.
//
// The spin-adapted form of the perturbative triples on spatial orbitals:
//   X_ijk^abc = sum_d (bd|ai) t_kj^cd - sum_l (ck|jl) t_il^ab
//   W_ijk^abc = X summed over the six simultaneous permutations of the pairs
//               (ia), (jb), (kc): twelve GEMMs per block of triples on the
//               tensor cores (hx_ccsd_triples in hx_engine.cu)
//   Z_ijk^abc = (jb|kc) t_i^a + (ia|kc) t_j^b + (ia|jb) t_k^c
//   Y_ijk^abc = 4 W_abc + W_bca + W_cab - 2 W_acb - 2 W_bac - 2 W_cba  (ijk fixed)
//   E[4] = sum W Y / (3 D),  E[5] = sum Z Y / (3 D),  D = e_i+e_j+e_k-e_a-e_b-e_c
// (k_t_energy), over the triples i <= j <= k, each weighted by its number of
// distinct permutations. E[4] + E[5] equals the spin-orbital (T) of the
// connected and disconnected triples amplitudes. One block per occupied
// triple, its threads over the v^3 virtual triples (32-bit index arithmetic).
#include <algorithm>

#include "hx_common.cuh"
#include "hx_kernels.h"

namespace {
constexpr int TNT = 256;

__device__ __forceinline__ double t_warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Bvv0[mu][(b d)] = C_mu,o+b C_mu,o+d ; Boo0[mu][(j l)] = C_mu,j C_mu,l
__global__ void k_t_pairs(const double *__restrict__ C, int N, int o, double *__restrict__ Bvv0,
                          double *__restrict__ Boo0)
{
    const int v = N - o;
    const long long nvv = (long long)N * v * v, noo = (long long)N * o * o;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nvv + noo;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < nvv) {
            const int mu = (int)(e / ((long long)v * v)), r = (int)(e % ((long long)v * v));
            Bvv0[e] = C[(long long)mu * N + o + r / v] * C[(long long)mu * N + o + r % v];
        } else {
            const long long f = e - nvv;
            const int mu = (int)(f / ((long long)o * o)), r = (int)(f % ((long long)o * o));
            Boo0[f] = C[(long long)mu * N + r / o] * C[(long long)mu * N + r % o];
        }
    }
}

// Per-block partials of E[4] and E[5] for one triple (i, j, k), i <= j <= k:
// the block's W_ijk^abc (v^3, [a][b][c]) sits in the slab at pair `blockIdx.x`;
// the triple counts w = 6, 3 or 1 times (its distinct permutations: the
// energy of a triple is unchanged by a simultaneous permutation of (ia),
// (jb), (kc)).
__global__ void __launch_bounds__(TNT) k_t_energy(const double *__restrict__ W, const int2 *__restrict__ pairs, int i,
                                                  const double *__restrict__ t1, const double *__restrict__ gov,
                                                  const double *__restrict__ Fmo, int N, int o, int v,
                                                  double *__restrict__ part)
{
    const int j = pairs[blockIdx.x].x, k = pairs[blockIdx.x].y;
    const int v2 = v * v, v3 = v2 * v;
    const long long ov = (long long)o * v;
    const double *Wb = W + (long long)blockIdx.x * v3;
    const double eijk = Fmo[(long long)i * N + i] + Fmo[(long long)j * N + j] + Fmo[(long long)k * N + k];
    const double wt = (i == j && j == k) ? 1.0 : ((i == j || j == k) ? 3.0 : 6.0);
    double e4 = 0.0, e5 = 0.0;
    for (int abc = threadIdx.x; abc < v3; abc += TNT) {
        const int c = abc % v, b = (abc / v) % v, a = abc / v2;
        const double w = Wb[abc];
        const double y = 4.0 * w + Wb[(c * v + a) * v + b] + Wb[(b * v + c) * v + a]
                       - 2.0 * Wb[(a * v + c) * v + b] - 2.0 * Wb[(b * v + a) * v + c] - 2.0 * Wb[(c * v + b) * v + a];
        const long long ia = (long long)i * v + a, jb = (long long)j * v + b, kc = (long long)k * v + c;
        const double z = gov[jb * ov + kc] * t1[ia] + gov[ia * ov + kc] * t1[jb] + gov[ia * ov + jb] * t1[kc];
        const double d = eijk - Fmo[(long long)(o + a) * N + o + a] - Fmo[(long long)(o + b) * N + o + b]
                       - Fmo[(long long)(o + c) * N + o + c];
        e4 += w * y / (3.0 * d);
        e5 += z * y / (3.0 * d);
    }
    __shared__ double sh[2][TNT / 32];
    e4 = t_warp_sum(e4);
    e5 = t_warp_sum(e5);
    if ((threadIdx.x & 31) == 0) { sh[0][threadIdx.x >> 5] = e4; sh[1][threadIdx.x >> 5] = e5; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s4 = 0.0, s5 = 0.0;
        for (int w = 0; w < TNT / 32; ++w) { s4 += sh[0][w]; s5 += sh[1][w]; }
        part[2 * (long long)blockIdx.x] = wt * s4;
        part[2 * (long long)blockIdx.x + 1] = wt * s5;
    }
}

// ordered sum of the block partials (deterministic)
__global__ void k_t_final(const double *__restrict__ part, long long nblk, double *__restrict__ out)
{
    __shared__ double sh[2][32];
    double s4 = 0.0, s5 = 0.0;
    for (long long b = threadIdx.x; b < nblk; b += 32) { s4 += part[2 * b]; s5 += part[2 * b + 1]; }
    sh[0][threadIdx.x] = s4;
    sh[1][threadIdx.x] = s5;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int t = 0; t < 32; ++t) { a += sh[0][t]; b += sh[1][t]; }
        out[0] = a;
        out[1] = b;
    }
}
}  // namespace

cudaError_t hx_triples_pairs(const double *C, int N, int o, double *Bvv0, double *Boo0, cudaStream_t s)
{
    const long long work = (long long)N * ((long long)(N - o) * (N - o) + (long long)o * o);
    const unsigned g = (unsigned)std::min<long long>((work + TNT - 1) / TNT, 4096);
    k_t_pairs<<<g, TNT, 0, s>>>(C, N, o, Bvv0, Boo0);
    hx_count_launches(1);
    return cudaGetLastError();
}

cudaError_t hx_triples_energy(const double *W, const int2 *pairs, int npairs, int i, const double *t1,
                              const double *gov, const double *Fmo, int N, int o, double *part, double *out,
                              cudaStream_t s)
{
    const int v = N - o;
    k_t_energy<<<(unsigned)npairs, TNT, 0, s>>>(W, pairs, i, t1, gov, Fmo, N, o, v, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_t_final<<<1, 32, 0, s>>>(part, npairs, out);
    hx_count_launches(2);
    return cudaGetLastError();
}
