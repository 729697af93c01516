// nqs_ed.cu -- exact diagonalisation of the kagome Heisenberg model in HBM.
//
// The memory-lean projecting Lanczos over the full 2^N basis (N <= 30):
//   w = H v                     k_heis_matvec   (bond masks, one state per thread)
//   w -= alpha v + beta v_prev  k_lz_orth       (alpha reduced from the matvec partials)
//   w = P w                     k_perm_sum x1-4 (sector projector, nibble bit-permute tables)
//   v_next = w / ||w||          k_lz_scale      (beta reduced from the projector partials)
// with the host holding only the tridiagonal (alpha, beta) and its lowest Ritz value.
//
// Upstream interfaces replaced:
//   kagome_heis_matvec                      src/nqs/nqs_lanczos.c:380-432
//   nqs_kagome_p6m_project_inplace          src/nqs/nqs_symproj.c:786-852
//   lanczos_smallest_projected_lean         src/mps/lanczos.c:824-960
//   lanczos_smallest_projected_lean_eigvec  src/mps/lanczos.c:972-1119
//   nqs_lanczos_e0_kagome_heisenberg_projected_lean[_eigvec]  src/nqs/nqs_lanczos.c:629-672
//
// The projector (1/G) sum_g chi(g) T(g) is evaluated, when chi is multiplicative on the
// group, as passes over a chain of subgroups and coset representatives (G = R1 H1,
// H1 = R2 H2, ...): 3 + 3 + 12 gathers per state for the 108-element p6m group of the
// 3 x 3 torus instead of 108.  Other character sets (the E irreps' traces) take the one-pass |G|-gather form.
// Reductions are block partials summed in a fixed order, so every run is deterministic
// and the eigenvector replay reproduces the first pass bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "nqs_internal.cuh"
#include "nqs/nqs_lanczos.h"
#include "nqs/nqs_symproj.h"

namespace nqs {
namespace {

constexpr int ED_THREADS = 256;
constexpr int ED_MAX_N = 30;
constexpr int ED_MAX_BONDS = 64;
constexpr int ED_NCH = 8;                 // 4-bit chunks of a 32-bit basis index
constexpr int ED_TAB = ED_NCH * 16;       // table entries per group element
constexpr int ED_SEED_RUN = 256;          // consecutive seed values per thread
constexpr size_t ED_MAX_SMEM = 200 * 1024;
constexpr double ED_BETA_MIN = 1e-14;     // src/mps/lanczos.c:919

// Bond masks; the first nlow touch one of the five lane bits (bits 0-4), the rest have
// both sites at bit 5 or above, where all 32 states of a warp agree.
struct Bonds {
    int nb, nlow;
    unsigned m[ED_MAX_BONDS];
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum in a fixed order, stored by thread 0 at part[blockIdx.x].
__device__ __forceinline__ void block_store(double v, double *part) {
    __shared__ double red[ED_THREADS / 32];
    v = warp_sum_d(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < ED_THREADS / 32; w++) t += red[w];
        part[blockIdx.x] = t;
    }
}

// Sum of np block partials in a fixed order, returned to every thread of the block.
__device__ __forceinline__ double block_total(const double *part, int np) {
    __shared__ double red[ED_THREADS / 32];
    __shared__ double tot;
    double v = 0.0;
    for (int i = threadIdx.x; i < np; i += ED_THREADS) v += part[i];
    v = warp_sum_d(v);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < ED_THREADS / 32; w++) t += red[w];
        tot = t;
    }
    __syncthreads();
    return tot;
}

// y = H x, H = J sum_b S_u.S_v: diagonal J/4 (nb - 2 n_anti) (a table indexed by n_anti),
// off-diagonal J/2 for every antiparallel bond (src/nqs/nqs_lanczos.c:380-432).  Within a
// warp the states differ in bits 0-4, so each bond's partner loads of a warp fall in one
// 256-byte segment.  GB300 issues an FP64 add for a whole warp at 16 cycles whatever its
// active lanes, so the bonds away from the lane bits -- where all 32 states of the warp
// agree -- are first collected into a warp-uniform bit mask and only the antiparallel ones
// are loaded (four at a time) and added.  part (may be null) receives the block partials
// of x.y.  popc >= 0 restricts to the states with that many set bits (down spins): the
// others are written as 0 without being evaluated.
__global__ void __launch_bounds__(ED_THREADS) k_heis_matvec(const double *__restrict__ x, double *__restrict__ y,
                                                            unsigned dim, Bonds B, double qJ, double hJ,
                                                            double *__restrict__ part, int popc) {
    __shared__ unsigned sm[ED_MAX_BONDS];
    __shared__ double diag[ED_MAX_BONDS + 1];
    for (int i = threadIdx.x; i < B.nb; i += ED_THREADS) sm[i] = B.m[i];
    for (int i = threadIdx.x; i <= B.nb; i += ED_THREADS) diag[i] = qJ * (double)(B.nb - 2 * i);
    __syncthreads();
    const int nb = B.nb, nlow = B.nlow;
    double dot = 0.0;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) {
        if (popc >= 0 && __popc(s) != popc) {
            // outside the magnetisation sector: H keeps the popcount, so x and H x are zero here
            y[s] = 0.0;
            continue;
        }
        double off = 0.0;
        int anti = 0;
#pragma unroll 4
        for (int b = 0; b < nlow; b++) {
            const unsigned m = sm[b];
            if (__popc(s & m) == 1) {
                off += __ldg(x + (s ^ m));
                anti++;
            }
        }
        uint64_t hm = 0;                                 // antiparallel high bonds (same in all lanes)
        for (int b = nlow; b < nb; b++) hm |= (uint64_t)(__popc(s & sm[b]) == 1) << (b - nlow);
        anti += __popcll(hm);
        while (hm) {
            double v[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                v[j] = 0.0;
                if (hm) {
                    const int b = __ffsll((long long)hm) - 1;
                    hm &= hm - 1;
                    v[j] = __ldg(x + (s ^ sm[nlow + b]));
                }
            }
            off += (v[0] + v[1]) + (v[2] + v[3]);
        }
        const double xs = __ldg(x + s);
        const double val = fma(diag[anti], xs, hJ * off);
        y[s] = val;
        dot = fma(xs, val, dot);
    }
    if (part) block_store(dot, part);
}

// y[s] = scale * sum_e chi[e] x[pi_e(s)] over m group elements, pi_e(s) = OR_c tab[e][c][nibble c
// of s] (bit i of pi_e(s) = bit perm_e[i] of s).  part (may be null) receives the block
// partials of y.y.  popc >= 0: states whose popcount differs are set to 0 (the permutations
// keep the popcount, so the sum for a state in the sector reads only states in it).
__global__ void __launch_bounds__(ED_THREADS) k_perm_sum(const double *__restrict__ x, double *__restrict__ y,
                                                         unsigned dim, int m, const unsigned *__restrict__ tab,
                                                         const double *__restrict__ chi, double scale,
                                                         double *__restrict__ part, int popc) {
    extern __shared__ __align__(16) unsigned char ed_smem[];
    double *s_chi = (double *)ed_smem;
    unsigned *s_tab = (unsigned *)(s_chi + m);
    for (int i = threadIdx.x; i < m; i += ED_THREADS) s_chi[i] = chi[i];
    for (int i = threadIdx.x; i < m * ED_TAB; i += ED_THREADS) s_tab[i] = tab[i];
    __syncthreads();
    double nrm = 0.0;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) {
        if (popc >= 0 && __popc(s) != popc) {
            y[s] = 0.0;                       // the magnetisation filter of the sector projector
            continue;
        }
        double acc = 0.0;
#pragma unroll 2
        for (int e = 0; e < m; e++) {
            const double c = s_chi[e];
            const unsigned *t = s_tab + e * ED_TAB;
            unsigned src = 0;
#pragma unroll
            for (int k = 0; k < ED_NCH; k++) src |= t[k * 16 + ((s >> (4 * k)) & 15u)];
            acc = fma(c, __ldg(x + src), acc);
        }
        const double v = acc * scale;
        y[s] = v;
        nrm = fma(v, v, nrm);
    }
    if (part) block_store(nrm, part);
}

// out bit i of A x = parity(rows[i] & x): one GF(2) matrix of 64 rows.
__device__ __forceinline__ uint64_t gf2_apply(const uint64_t *rows, uint64_t x) {
    uint64_t r = 0;
#pragma unroll 8
    for (int i = 0; i < 64; i++) r |= (uint64_t)(__popcll(rows[i] & x) & 1) << i;
    return r;
}

// v[i] = u_i - 1/2 with u_i the (i+1)-th xorshift64 (13, 7, 17) output from x0, >> 11,
// times 2^-53 (src/mps/lanczos.c:864-870).  Thread c starts ED_SEED_RUN * c steps in by
// the jump matrices jump[j] = M^(ED_SEED_RUN * 2^j) of the step map M.
__global__ void __launch_bounds__(ED_THREADS) k_lz_seed(double *__restrict__ v, unsigned dim, uint64_t x0,
                                                        const uint64_t *__restrict__ jump, int nj) {
    __shared__ uint64_t sj[32 * 64];
    for (int i = threadIdx.x; i < nj * 64; i += ED_THREADS) sj[i] = jump[i];
    __syncthreads();
    const unsigned c = blockIdx.x * ED_THREADS + threadIdx.x;
    const uint64_t first = (uint64_t)c * ED_SEED_RUN;
    if (first >= dim) return;
    uint64_t x = x0;
    for (int j = 0; j < nj; j++)
        if ((c >> j) & 1u) x = gf2_apply(sj + 64 * j, x);
    const unsigned n = (unsigned)min((uint64_t)ED_SEED_RUN, (uint64_t)dim - first);
    for (unsigned i = 0; i < n; i++) {
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        v[first + i] = (double)(x >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
}

// w -= alpha v (+ beta_k v_prev for k > 0); alpha = sum of the matvec partials, stored in
// al[k] by block 0 (src/mps/lanczos.c:903-912).
__global__ void __launch_bounds__(ED_THREADS) k_lz_orth(double *__restrict__ w, const double *__restrict__ v,
                                                        const double *__restrict__ vp, unsigned dim,
                                                        const double *__restrict__ part, int np, double *al,
                                                        const double *be, int k) {
    const double a = block_total(part, np);
    if (blockIdx.x == 0 && threadIdx.x == 0) al[k] = a;
    const double b = k > 0 ? be[k] : 0.0;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) {
        double t = fma(-a, v[s], w[s]);
        if (k > 0) t = fma(-b, vp[s], t);
        w[s] = t;
    }
}

// beta = sqrt(sum of the projector partials), stored in be[k+1] by block 0; unless beta is
// below the breakdown bound, w *= 1/beta (src/mps/lanczos.c:945-947) and acc += z w.
__global__ void __launch_bounds__(ED_THREADS) k_lz_scale(double *__restrict__ w, unsigned dim,
                                                         const double *__restrict__ part, int np, double *be,
                                                         int k, double *__restrict__ acc, double z) {
    const double b = sqrt(block_total(part, np));
    if (blockIdx.x == 0 && threadIdx.x == 0) be[k + 1] = b;
    if (!(b >= ED_BETA_MIN)) return;
    const double inv = 1.0 / b;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) {
        const double t = w[s] * inv;
        w[s] = t;
        if (acc) acc[s] = fma(z, t, acc[s]);
    }
}

// n = sqrt(sum of partials) -> *nout; v /= n when n > 0 (src/mps/lanczos.c:884); acc = z v.
__global__ void __launch_bounds__(ED_THREADS) k_lz_normalise(double *__restrict__ v, unsigned dim,
                                                             const double *__restrict__ part, int np,
                                                             double *nout, double *__restrict__ acc, double z) {
    const double n = sqrt(block_total(part, np));
    if (blockIdx.x == 0 && threadIdx.x == 0) *nout = n;
    if (!(n > 0.0)) return;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) {
        const double t = v[s] / n;
        v[s] = t;
        if (acc) acc[s] = z * t;
    }
}

// Block partials of x.x.
__global__ void __launch_bounds__(ED_THREADS) k_sumsq(const double *__restrict__ x, unsigned dim,
                                                      double *__restrict__ part) {
    double t = 0.0;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) t = fma(x[s], x[s], t);
    block_store(t, part);
}

// x *= 1 / ||x|| when ||x|| > 0 (src/mps/lanczos.c:1104-1105).
__global__ void __launch_bounds__(ED_THREADS) k_unit(double *__restrict__ x, unsigned dim,
                                                     const double *__restrict__ part, int np) {
    const double n = sqrt(block_total(part, np));
    if (!(n > 0.0)) return;
    const double inv = 1.0 / n;
    const unsigned stride = gridDim.x * ED_THREADS;
    for (unsigned s = blockIdx.x * ED_THREADS + threadIdx.x; s < dim; s += stride) x[s] *= inv;
}

// ------------------------------------------------------------------------ host side

// Kagome bonds in the loop order of src/nqs/nqs_lanczos.c:386-431: per cell the up
// triangle (A,B), (A,C), (B,C); the down triangle (A,B-), (A,C-), (B-,C-) with
// B- = B(cx-1, cy), C- = C(cx, cy-1), wrapped with PBC, skipped on the open edges.
bool kagome_bonds(int Lx, int Ly, int pbc, Bonds &B) {
    B.nb = 0;
    auto site = [&](int cx, int cy, int sub) { return 3 * (cx * Ly + cy) + sub; };
    auto add = [&](int u, int v) {
        if (B.nb >= ED_MAX_BONDS) return false;
        B.m[B.nb++] = (1u << u) | (1u << v);
        return true;
    };
    B.nlow = 0;
    for (int cx = 0; cx < Lx; cx++)
        for (int cy = 0; cy < Ly; cy++) {
            int A = site(cx, cy, 0), Bs = site(cx, cy, 1), Cs = site(cx, cy, 2);
            if (!add(A, Bs) || !add(A, Cs) || !add(Bs, Cs)) return false;
            int cxm, cym;
            if (pbc) {
                cxm = (cx - 1 + Lx) % Lx;
                cym = (cy - 1 + Ly) % Ly;
            } else if (cx == 0 || cy == 0) {
                continue;
            } else {
                cxm = cx - 1;
                cym = cy - 1;
            }
            int Bm = site(cxm, cy, 1), Cm = site(cx, cym, 2);
            if (!add(A, Bm) || !add(A, Cm) || !add(Bm, Cm)) return false;
        }
    // lane-bit bonds first (a stable partition keeps the loop order within each group)
    std::stable_partition(B.m, B.m + B.nb, [](unsigned m) { return (m & 31u) != 0; });
    while (B.nlow < B.nb && (B.m[B.nlow] & 31u)) B.nlow++;
    return true;
}

// ---- sector projector plan
constexpr int ED_MAX_PASSES = 4;

struct ProjPlan {
    int N = 0, G = 0, passes = 0;
    int size[ED_MAX_PASSES] = {0, 0, 0, 0};
    std::vector<int> elems;          // pass 0 elements, then pass 1, ...
    std::vector<int> key_perm;
    std::vector<double> key_chars;
    DevBuf<unsigned> tab;            // [elems][ED_NCH][16] in elems order
    DevBuf<double> chi;              // [elems] in elems order
};

// Smallest d + G/d over the divisors 1 < d < G (G when G is prime or small).
int best_split_cost(int G) {
    int best = G;
    for (int d = 2; d < G; d++)
        if (G % d == 0) best = std::min(best, d + G / d);
    return best;
}

// Best split of the group grp (element indices, closed under mul, G x G table) into a
// subgroup H generated by one or two elements and left-coset representatives R (every
// element of grp exactly once as r o h) with |H| + |R| minimal; false when no split makes
// |H| + |R| < |grp|.
bool split_group(const std::vector<int> &grp, const std::vector<int> &mul, int G, std::vector<int> &Hout,
                 std::vector<int> &Rout) {
    const int n = (int)grp.size();
    const int target = best_split_cost(n);
    if (target >= n) return false;
    int best_cost = n;
    std::vector<int> best, H;
    std::vector<char> in(G);
    auto closure = [&](int g1, int g2) {
        std::fill(in.begin(), in.end(), 0);
        H.clear();
        int gens[2] = {g1, g2};
        int ng = g2 < 0 ? 1 : 2;
        for (int i = 0; i < ng; i++)
            if (!in[gens[i]]) {
                in[gens[i]] = 1;
                H.push_back(gens[i]);
            }
        for (size_t q = 0; q < H.size(); q++)
            for (int i = 0; i < ng; i++) {
                int c = mul[(size_t)H[q] * G + gens[i]];
                if (!in[c]) {
                    in[c] = 1;
                    H.push_back(c);
                }
            }
    };
    auto consider = [&]() {
        int h = (int)H.size();
        if (h <= 1 || h >= n || n % h) return;
        if (h + n / h < best_cost) {
            best_cost = h + n / h;
            best = H;
        }
    };
    for (int i = 0; i < n && best_cost > target; i++) {
        closure(grp[i], -1);
        consider();
    }
    for (int i = 0; i < n && best_cost > target; i++)
        for (int j = i + 1; j < n && best_cost > target; j++) {
            closure(grp[i], grp[j]);
            consider();
        }
    if (best_cost >= n) return false;
    std::vector<char> cov(G, 0);
    std::vector<int> R;
    for (int g : grp) {
        if (cov[g]) continue;
        R.push_back(g);
        for (int h : best) {
            int c = mul[(size_t)g * G + h];
            if (cov[c]) return false;                   // not a partition
            cov[c] = 1;
        }
    }
    if (R.size() * best.size() != (size_t)n) return false;
    Hout = best;
    Rout = R;
    return true;
}

// Host plan (no device work): validates the table and picks the factorisation.
bool plan_host(int N, int G, const int *perm, const double *chars, ProjPlan &P) {
    if (N <= 0 || N > ED_MAX_N || G <= 0 || !perm || !chars) {
        set_error("invalid projector arguments (N=%d, G=%d)", N, G);
        return false;
    }
    for (int g = 0; g < G; g++) {
        std::vector<char> seen(N, 0);
        for (int i = 0; i < N; i++) {
            int j = perm[(size_t)g * N + i];
            if (j < 0 || j >= N || seen[j]) {
                set_error("perm row %d is not a permutation of 0..%d", g, N - 1);
                return false;
            }
            seen[j] = 1;
        }
        if (!std::isfinite(chars[g])) {
            set_error("character %d is not finite", g);
            return false;
        }
    }
    P.N = N;
    P.G = G;
    P.passes = 1;
    for (int k = 0; k < ED_MAX_PASSES; k++) P.size[k] = 0;
    P.size[0] = G;
    P.elems.resize(G);
    for (int g = 0; g < G; g++) P.elems[g] = g;
    auto drop_zero_characters = [&]() {              // the one-pass form skips chi = 0
        P.elems.clear();
        for (int g = 0; g < G; g++)
            if (chars[g] != 0.0) P.elems.push_back(g);
        P.size[0] = (int)P.elems.size();
        return true;
    };
    if (best_split_cost(G) >= G) return drop_zero_characters();

    // Row lookup by content (rows are permutations of N <= 30 sites: hash by a 64-bit mix).
    auto row_hash = [&](const int *r) {
        uint64_t h = 1469598103934665603ull;
        for (int i = 0; i < N; i++) h = (h ^ (uint64_t)(r[i] + 1)) * 1099511628211ull;
        return h;
    };
    std::vector<std::pair<uint64_t, int>> index(G);
    for (int g = 0; g < G; g++) index[g] = {row_hash(perm + (size_t)g * N), g};
    std::sort(index.begin(), index.end());
    std::vector<int> tmp(N);
    // element whose row is perm_a o perm_b (row[i] = perm_a[perm_b[i]]), or -1
    auto compose = [&](int a, int b) {
        const int *pa = perm + (size_t)a * N, *pb = perm + (size_t)b * N;
        for (int i = 0; i < N; i++) tmp[i] = pa[pb[i]];
        uint64_t h = row_hash(tmp.data());
        auto it = std::lower_bound(index.begin(), index.end(), std::make_pair(h, -1));
        for (; it != index.end() && it->first == h; ++it)
            if (std::equal(tmp.begin(), tmp.end(), perm + (size_t)it->second * N)) return it->second;
        return -1;
    };
    auto close_to = [](double a, double b) { return std::fabs(a - b) <= 1e-12 * std::max(1.0, std::fabs(a)); };
    // The table must be a group with chi multiplicative on it; otherwise stay direct.
    std::vector<int> mul((size_t)G * G);
    for (int a = 0; a < G; a++)
        for (int b = 0; b < G; b++) {
            int c = compose(a, b);
            if (c < 0 || !close_to(chars[c], chars[a] * chars[b])) return drop_zero_characters();
            mul[(size_t)a * G + b] = c;
        }
    // Peel subgroups: G = R1 H1, H1 = R2 H2, ...; passes run H_k, R_k, ..., R1.
    std::vector<int> cur(G);
    for (int g = 0; g < G; g++) cur[g] = g;
    std::vector<std::vector<int>> outer;
    std::vector<int> H, R;
    while ((int)outer.size() < ED_MAX_PASSES - 1 && split_group(cur, mul, G, H, R)) {
        outer.push_back(R);
        cur = H;
    }
    if (outer.empty()) return drop_zero_characters();
    P.passes = 1 + (int)outer.size();
    P.elems = cur;
    P.size[0] = (int)cur.size();
    for (int k = 0; k < (int)outer.size(); k++) {
        const std::vector<int> &r = outer[outer.size() - 1 - k];
        P.size[k + 1] = (int)r.size();
        P.elems.insert(P.elems.end(), r.begin(), r.end());
    }
    return true;
}

ProjPlan &plan_cache() {
    static ProjPlan p;
    return p;
}

// Device plan for (N, G, perm, chars), rebuilt only when the table changes.
ProjPlan *plan_get(int N, int G, const int *perm, const double *chars) {
    ProjPlan &P = plan_cache();
    size_t np = (size_t)N * G;
    if (P.N == N && P.G == G && P.key_perm.size() == np && P.tab.p &&
        std::equal(P.key_perm.begin(), P.key_perm.end(), perm) &&
        std::equal(P.key_chars.begin(), P.key_chars.end(), chars))
        return &P;
    P.N = 0;
    if (!plan_host(N, G, perm, chars, P)) return nullptr;
    for (int p = 0; p < P.passes; p++)
        if ((size_t)P.size[p] * (ED_TAB * sizeof(unsigned) + sizeof(double)) > ED_MAX_SMEM) {
            set_error("sector projector pass of %d elements exceeds shared memory", P.size[p]);
            P.N = 0;
            return nullptr;
        }
    const int ne = (int)P.elems.size();               // |H| + |R|, or G for the direct form
    std::vector<unsigned> tab((size_t)ne * ED_TAB, 0u);
    std::vector<double> chi(ne);
    for (int e = 0; e < ne; e++) {
        const int g = P.elems[e];
        const int *pg = perm + (size_t)g * N;
        std::vector<int> pinv(N);
        for (int i = 0; i < N; i++) pinv[pg[i]] = i;
        unsigned *t = tab.data() + (size_t)e * ED_TAB;
        for (int c = 0; c < ED_NCH; c++)
            for (int v = 0; v < 16; v++) {
                unsigned m = 0;
                for (int b = 0; b < 4; b++) {
                    int j = 4 * c + b;
                    if (((v >> b) & 1) && j < N) m |= 1u << pinv[j];
                }
                t[c * 16 + v] = m;
            }
        chi[e] = chars[g];
    }
    if (!P.tab.ensure(tab.size()) || !P.chi.ensure(ne) ||
        !NQS_CUDA(cudaMemcpy(P.tab.p, tab.data(), tab.size() * sizeof(unsigned), cudaMemcpyHostToDevice)) ||
        !NQS_CUDA(cudaMemcpy(P.chi.p, chi.data(), ne * sizeof(double), cudaMemcpyHostToDevice))) {
        P.N = 0;
        return nullptr;
    }
    P.key_perm.assign(perm, perm + np);
    P.key_chars.assign(chars, chars + G);
    return &P;
}

int ed_grid(unsigned dim) {
    long want = ((long)dim + ED_THREADS - 1) / ED_THREADS;
    long cap = (long)ctx().sm_count * (2048 / ED_THREADS);
    return (int)std::max(1L, std::min(want, cap));
}

bool launch_perm_pass(const ProjPlan &P, int pass, const double *x, double *y, unsigned dim, double scale,
                      double *part, cudaStream_t st, int popc = -1) {
    static bool attr = false;
    if (!attr) {
        if (!NQS_CUDA(cudaFuncSetAttribute(k_perm_sum, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)ED_MAX_SMEM)))
            return false;
        attr = true;
    }
    int off = 0;
    for (int k = 0; k < pass; k++) off += P.size[k];
    const int m = P.size[pass];
    const size_t smem = (size_t)m * (ED_TAB * sizeof(unsigned) + sizeof(double));
    NQS_LAUNCH("ed_project_pass");
    k_perm_sum<<<ed_grid(dim), ED_THREADS, smem, st>>>(x, y, dim, m, P.tab.p + (size_t)off * ED_TAB,
                                                       P.chi.p + off, scale, part, popc);
    return NQS_CUDA(cudaGetLastError());
}

// Projects *a in place (using *t as scratch; the pointers may be swapped so that the
// result is in *a).  part (may be null) receives the partials of the result's norm.
bool project(const ProjPlan &P, double *&a, double *&t, unsigned dim, double *part, cudaStream_t st,
             int popc = -1) {
    const double invG = 1.0 / (double)P.G;
    for (int k = 0; k < P.passes; k++) {
        const bool last = k + 1 == P.passes;
        if (!launch_perm_pass(P, k, a, t, dim, last ? invG : 1.0, last ? part : nullptr, st, popc)) return false;
        std::swap(a, t);
    }
    return true;
}

// ---- seed
struct Gf2 {
    uint64_t r[64];
};

Gf2 gf2_mul(const Gf2 &A, const Gf2 &B) {   // (A B) x = A (B x)
    Gf2 C;
    for (int i = 0; i < 64; i++) {
        uint64_t acc = 0;
        for (int j = 0; j < 64; j++)
            if ((A.r[i] >> j) & 1ull) acc ^= B.r[j];
        C.r[i] = acc;
    }
    return C;
}

// jump[j] = M^(ED_SEED_RUN 2^j), M the xorshift64 (13, 7, 17) step map.
const std::vector<uint64_t> &seed_jumps() {
    static std::vector<uint64_t> J;
    if (!J.empty()) return J;
    Gf2 M{};
    for (int j = 0; j < 64; j++) {
        uint64_t x = 1ull << j;
        x ^= x << 13;
        x ^= x >> 7;
        x ^= x << 17;
        for (int i = 0; i < 64; i++)
            if ((x >> i) & 1ull) M.r[i] |= 1ull << j;
    }
    Gf2 P = M;
    for (int run = 1; run < ED_SEED_RUN; run *= 2) P = gf2_mul(P, P);
    for (int j = 0; j < 32; j++) {
        J.insert(J.end(), P.r, P.r + 64);
        P = gf2_mul(P, P);
    }
    return J;
}

struct SeedDev {
    DevBuf<uint64_t> jump;
};

bool launch_seed(double *v, unsigned dim, int alternate, cudaStream_t st, uint64_t state = 0) {
    static SeedDev sd;
    const auto &J = seed_jumps();
    if (!sd.jump.p) {
        if (!sd.jump.ensure(J.size()) ||
            !NQS_CUDA(cudaMemcpy(sd.jump.p, J.data(), J.size() * sizeof(uint64_t), cudaMemcpyHostToDevice)))
            return false;
    }
    const unsigned threads = (unsigned)(((uint64_t)dim + ED_SEED_RUN - 1) / ED_SEED_RUN);
    int nj = 0;
    while (nj < 32 && (threads - 1) >> nj) nj++;
    const uint64_t x0 = state ? state : (alternate ? 0xBEEFBABEull : 0xA5A5A5A5A5A5A5A5ull) ^ (uint64_t)dim;
    NQS_LAUNCH("ed_seed");
    k_lz_seed<<<(threads + ED_THREADS - 1) / ED_THREADS, ED_THREADS, 0, st>>>(v, dim, x0, sd.jump.p, nj);
    return NQS_CUDA(cudaGetLastError());
}

// ---- tridiagonal helpers (host)
// Lowest eigenvalue of the symmetric tridiagonal (a[0..k-1], off-diagonal b[0..k-2]) by
// Sturm-sequence bisection to the bracket's rounding limit.
double tri_lowest(const double *a, const double *b, int k) {
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < k; i++) {
        double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < k ? std::fabs(b[i]) : 0.0);
        lo = std::min(lo, a[i] - r);
        hi = std::max(hi, a[i] + r);
    }
    for (int it = 0; it < 256; it++) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        int neg = 0;
        double q = 1.0;
        for (int i = 0; i < k; i++) {
            q = a[i] - mid - (i > 0 ? b[i - 1] * b[i - 1] / q : 0.0);
            if (q == 0.0) q = -1e-300;
            if (q < 0.0) neg++;
        }
        if (neg >= 1) hi = mid;
        else lo = mid;
    }
    return 0.5 * (lo + hi);
}

// Unit eigenvector of the tridiagonal for eigenvalue lam: inverse iteration on (T - lam I)
// with a partially pivoted tridiagonal LU (three sweeps from a constant start).
std::vector<double> tri_vector(const double *a, const double *b, int k, double lam) {
    std::vector<double> z(k, 1.0);
    if (k == 1) return z;
    const double tiny = 1e-300 + 1e-15 * (std::fabs(lam) + 1.0);
    for (int sweep = 0; sweep < 3; sweep++) {
        // rows i: (l_i, d_i, u_i) with band d, u, u2 after pivoting
        std::vector<double> d(k), u(k, 0.0), u2(k, 0.0), l(k, 0.0), rhs = z;
        for (int i = 0; i < k; i++) {
            d[i] = a[i] - lam;
            if (i + 1 < k) u[i] = b[i];
            if (i > 0) l[i] = b[i - 1];
        }
        for (int i = 0; i + 1 < k; i++) {
            if (std::fabs(l[i + 1]) > std::fabs(d[i])) {    // swap rows i and i+1
                std::swap(d[i], l[i + 1]);
                std::swap(u[i], d[i + 1]);
                std::swap(u2[i], u[i + 1]);
                std::swap(rhs[i], rhs[i + 1]);
            }
            if (d[i] == 0.0) d[i] = tiny;
            double f = l[i + 1] / d[i];
            d[i + 1] -= f * u[i];
            u[i + 1] -= f * u2[i];
            rhs[i + 1] -= f * rhs[i];
            l[i + 1] = 0.0;
        }
        if (d[k - 1] == 0.0) d[k - 1] = tiny;
        for (int i = k - 1; i >= 0; i--) {
            double s = rhs[i];
            if (i + 1 < k) s -= u[i] * rhs[i + 1];
            if (i + 2 < k) s -= u2[i] * rhs[i + 2];
            rhs[i] = s / d[i];
        }
        double n = 0.0;
        for (double x : rhs) n += x * x;
        n = std::sqrt(n);
        if (!(n > 0.0) || !std::isfinite(n)) break;
        for (int i = 0; i < k; i++) z[i] = rhs[i] / n;
    }
    return z;
}

// ---- the Lanczos run
struct EdVecs {
    DevBuf<double> v[4];
    DevBuf<double> acc;
    DevBuf<double> part, al, be, nrm;
};

std::vector<double> &last_alpha() {
    static std::vector<double> a;
    return a;
}
std::vector<double> &last_beta() {
    static std::vector<double> b;
    return b;
}

struct LeanOut {
    double lambda = 0.0, prev = 0.0;
    int iters = 0, converged = 0;
};

// popc >= 0: the magnetisation sector (states with popc set bits), filtered inside every
// matvec and projection.  seed_state != 0: the seed protocol of the upstream sector drivers
// (scripts/research_kagome_sz_spatial.c:206-236, research_kagome_spin_gap.c:122-143): the
// xorshift64 seed from that state is projected and normalised, then handed to the lean
// Lanczos as its initial vector, which projects and normalises it again.
int lanczos_kagome(int Lx, int Ly, double J, int pbc, const int *perm, const double *chars, int G, int max_iters,
                   double tol, double *out_eig, double *out_vec, lanczos_result_t *out_res, int popc = -1,
                   uint64_t seed_state = 0) {
    clear_error();
    if (out_res) *out_res = lanczos_result_t{0.0, 0, 0, 0.0};
    const int N = 3 * Lx * Ly;
    if (Lx <= 0 || Ly <= 0 || N > ED_MAX_N || !perm || !chars || G <= 0 || max_iters <= 0 || !out_eig) {
        set_error("invalid Lanczos arguments");
        return -1;
    }
    if (!ensure_context()) return -1;
    cudaStream_t st = ctx().stream;
    Bonds B;
    if (!kagome_bonds(Lx, Ly, pbc, B)) {
        set_error("too many bonds");
        return -1;
    }
    ProjPlan *P = plan_get(N, G, perm, chars);
    if (!P) return -1;
    const unsigned dim = 1u << N;
    if ((long)max_iters > (long)dim) max_iters = (int)dim;
    const int grid = ed_grid(dim);
    const size_t need = dim;
    EdVecs E;
    for (auto &b : E.v)
        if (!b.ensure(need)) return -1;
    if ((out_vec && !E.acc.ensure(need)) || !E.part.ensure(grid) || !E.al.ensure(max_iters + 1) ||
        !E.be.ensure(max_iters + 2) || !E.nrm.ensure(1))
        return -1;
    if (!NQS_CUDA(cudaMemsetAsync(E.be.p, 0, sizeof(double) * (max_iters + 2), st))) return -1;
    const double qJ = 0.25 * J, hJ = 0.5 * J;
    double *vc = E.v[0].p, *vp = E.v[1].p, *w = E.v[2].p, *t = E.v[3].p;

    // seed -> project -> normalise (again from the alternate seed when the projection
    // leaves nothing, src/mps/lanczos.c:874-884); acc = z0 v0 on the replay
    int alt_used = 0;
    auto make_seed = [&](int alt, double *acc, double z0, double *norm_out) -> bool {
        if (!launch_seed(vc, dim, alt, st, alt ? 0 : seed_state) || !project(*P, vc, t, dim, E.part.p, st, popc))
            return false;
        if (seed_state && !alt) {
            // the caller-built seed: normalised once before the Lanczos projects it again
            NQS_LAUNCH("ed_normalise");
            k_lz_normalise<<<grid, ED_THREADS, 0, st>>>(vc, dim, E.part.p, grid, E.nrm.p, nullptr, 0.0);
            if (!NQS_CUDA(cudaGetLastError()) || !project(*P, vc, t, dim, E.part.p, st, popc)) return false;
        }
        {
            NQS_LAUNCH("ed_normalise");
            k_lz_normalise<<<grid, ED_THREADS, 0, st>>>(vc, dim, E.part.p, grid, E.nrm.p, acc, z0);
        }
        if (!NQS_CUDA(cudaGetLastError())) return false;
        return NQS_CUDA(cudaMemcpyAsync(norm_out, E.nrm.p, sizeof(double), cudaMemcpyDeviceToHost, st)) &&
               NQS_CUDA(cudaStreamSynchronize(st));
    };
    auto step = [&](int k, bool with_scale, double *acc, double z) -> bool {
        {
            NQS_LAUNCH("ed_matvec");
            k_heis_matvec<<<grid, ED_THREADS, 0, st>>>(vc, w, dim, B, qJ, hJ, E.part.p, popc);
        }
        {
            NQS_LAUNCH("ed_orth");
            k_lz_orth<<<grid, ED_THREADS, 0, st>>>(w, vc, vp, dim, E.part.p, grid, E.al.p, E.be.p, k);
        }
        if (!NQS_CUDA(cudaGetLastError()) || !project(*P, w, t, dim, E.part.p, st, popc)) return false;
        if (with_scale) {
            NQS_LAUNCH("ed_scale");
            k_lz_scale<<<grid, ED_THREADS, 0, st>>>(w, dim, E.part.p, grid, E.be.p, k, acc, z);
        }
        return NQS_CUDA(cudaGetLastError());
    };
    auto rotate = [&]() {
        double *old = vp;
        vp = vc;
        vc = w;
        w = old;
    };

    double n0 = 0.0;
    if (!make_seed(0, nullptr, 0.0, &n0)) return -1;
    if (n0 < 1e-14) {
        alt_used = 1;
        if (!make_seed(1, nullptr, 0.0, &n0)) return -1;
    }
    std::vector<double> al(max_iters + 1, 0.0), be(max_iters + 2, 0.0);
    LeanOut o;
    int K = 0;
    for (int k = 0; k < max_iters; k++) {
        if (!step(k, true, nullptr, 0.0)) return -1;
        double ab[2];
        if (!NQS_CUDA(cudaMemcpyAsync(&ab[0], E.al.p + k, sizeof(double), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaMemcpyAsync(&ab[1], E.be.p + k + 1, sizeof(double), cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaStreamSynchronize(st)))
            return -1;
        al[k] = ab[0];
        be[k + 1] = ab[1];
        K = k + 1;
        if (!(ab[1] >= ED_BETA_MIN)) break;
        o.prev = o.lambda;
        o.lambda = tri_lowest(al.data(), be.data() + 1, K);
        if (k > 5 && std::fabs(o.lambda - o.prev) < tol) {
            o.converged = 1;
            break;
        }
        rotate();
    }
    o.iters = K;
    last_alpha().assign(al.begin(), al.begin() + K);
    last_beta().assign(be.begin(), be.begin() + K + 1);

    if (!out_vec) {
        *out_eig = o.lambda;
        if (out_res) {
            out_res->eigenvalue = o.lambda;
            out_res->iterations = K;
            out_res->converged = o.converged;
            out_res->residual_norm = K > 0 ? std::fabs(o.lambda - o.prev) : 0.0;
        }
        return 0;
    }

    // Eigenvector: lowest pair of the K x K tridiagonal, then the replay
    // (src/mps/lanczos.c:1057-1105).
    const double lam = tri_lowest(al.data(), be.data() + 1, K);
    std::vector<double> z = tri_vector(al.data(), be.data() + 1, K, lam);
    vc = E.v[0].p;
    vp = E.v[1].p;
    w = E.v[2].p;
    t = E.v[3].p;
    double nr = 0.0;
    if (!make_seed(alt_used, E.acc.p, z[0], &nr)) return -1;
    for (int k = 0; k + 1 < K; k++) {
        if (!(be[k + 1] >= ED_BETA_MIN)) break;
        if (!step(k, true, E.acc.p, z[k + 1])) return -1;
        rotate();
    }
    {
        NQS_LAUNCH("ed_normalise");
        k_sumsq<<<grid, ED_THREADS, 0, st>>>(E.acc.p, dim, E.part.p);
        k_unit<<<grid, ED_THREADS, 0, st>>>(E.acc.p, dim, E.part.p, grid);
    }
    if (!NQS_CUDA(cudaGetLastError()) ||
        !NQS_CUDA(cudaMemcpyAsync(out_vec, E.acc.p, sizeof(double) * (size_t)dim, cudaMemcpyDeviceToHost, st)) ||
        !NQS_CUDA(cudaStreamSynchronize(st)))
        return -1;
    *out_eig = lam;
    if (out_res) {
        out_res->eigenvalue = lam;
        out_res->iterations = K;
        out_res->converged = (K >= 6 && std::fabs(lam - o.prev) < tol) ? 1 : 0;
        out_res->residual_norm = K >= 2 ? std::fabs(lam - o.prev) : 0.0;
    }
    return 0;
}

}  // namespace
}  // namespace nqs

using namespace nqs;

extern "C" {

int nqs_lanczos_e0_kagome_heisenberg_projected_lean(int Lx, int Ly, double J, int pbc, const int *perm,
                                                    const double *chars, int G, int max_iters, double tol,
                                                    double *out_eig, lanczos_result_t *out_res) {
    return lanczos_kagome(Lx, Ly, J, pbc, perm, chars, G, max_iters, tol, out_eig, nullptr, out_res);
}

int nqs_lanczos_e0_kagome_heisenberg_projected_lean_eigvec(int Lx, int Ly, double J, int pbc, const int *perm,
                                                           const double *chars, int G, int max_iters,
                                                           double tol, double *out_eig, double *out_vec,
                                                           lanczos_result_t *out_res) {
    if (!out_vec) {
        set_error("out_eigenvector is required");
        return -1;
    }
    return lanczos_kagome(Lx, Ly, J, pbc, perm, chars, G, max_iters, tol, out_eig, out_vec, out_res);
}

int nqs_gpu_lanczos_e0_kagome_sz_projected_lean(int Lx, int Ly, double J, int pbc, const int *perm,
                                                const double *chars, int G, int popcount,
                                                unsigned long long seed_state, int max_iters, double tol,
                                                double *out_eig, double *out_vec, lanczos_result_t *out_res) {
    const int N = 3 * Lx * Ly;
    if (popcount < -1 || popcount > N) {
        clear_error();
        set_error("popcount %d out of range for N = %d", popcount, N);
        return -1;
    }
    return lanczos_kagome(Lx, Ly, J, pbc, perm, chars, G, max_iters, tol, out_eig, out_vec, out_res, popcount,
                          (uint64_t)seed_state);
}

int nqs_gpu_kagome_heis_matvec(int Lx, int Ly, double J, int pbc, const double *d_in, double *d_out) {
    clear_error();
    const int N = 3 * Lx * Ly;
    if (Lx <= 0 || Ly <= 0 || N > ED_MAX_N || !d_in || !d_out || d_in == d_out) {
        set_error("invalid matvec arguments");
        return -1;
    }
    if (!ensure_context()) return -1;
    Bonds B;
    if (!kagome_bonds(Lx, Ly, pbc, B)) return -1;
    const unsigned dim = 1u << N;
    {
        NQS_LAUNCH("ed_matvec");
        k_heis_matvec<<<ed_grid(dim), ED_THREADS, 0, ctx().stream>>>(d_in, d_out, dim, B, 0.25 * J, 0.5 * J,
                                                                     nullptr, -1);
    }
    return NQS_CUDA(cudaGetLastError()) ? 0 : -1;
}

int nqs_gpu_sector_project(int N, int G, const int *perm, const double *chars, const double *d_in,
                           double *d_out) {
    clear_error();
    if (!d_in || !d_out) {
        set_error("invalid projector arguments");
        return -1;
    }
    if (!ensure_context()) return -1;
    ProjPlan *P = plan_get(N, G, perm, chars);
    if (!P) return -1;
    const unsigned dim = 1u << N;
    cudaStream_t st = ctx().stream;
    static DevBuf<double> tmp[2];
    if (!tmp[0].ensure(dim) || (P->passes > 2 && !tmp[1].ensure(dim))) return -1;
    const double invG = 1.0 / (double)G;
    const double *src = d_in;
    for (int k = 0; k < P->passes; k++) {
        const bool last = k + 1 == P->passes;
        double *dst = last ? d_out : tmp[k % 2].p;
        if (dst == src) dst = tmp[0].p;              // a single pass in place: copied back below
        if (!launch_perm_pass(*P, k, src, dst, dim, last ? invG : 1.0, nullptr, st)) return -1;
        src = dst;
    }
    if (src != d_out &&
        !NQS_CUDA(cudaMemcpyAsync(d_out, src, sizeof(double) * dim, cudaMemcpyDeviceToDevice, st)))
        return -1;
    return 0;
}

int nqs_gpu_lanczos_seed(int N, int alternate, double *d_out) {
    clear_error();
    if (N <= 0 || N > ED_MAX_N || !d_out) {
        set_error("invalid seed arguments");
        return -1;
    }
    if (!ensure_context()) return -1;
    return launch_seed(d_out, 1u << N, alternate, ctx().stream) ? 0 : -1;
}

int nqs_gpu_lanczos_last_coeffs(int cap, double *alpha, double *beta) {
    const auto &a = last_alpha();
    const auto &b = last_beta();
    const int K = (int)a.size();
    for (int i = 0; i < K && i < cap; i++)
        if (alpha) alpha[i] = a[i];
    for (int i = 0; i <= K && i <= cap; i++)
        if (beta) beta[i] = i == 0 ? 0.0 : b[i];
    return K;
}

int nqs_ed_projector_plan(int N, int G, const int *perm, const double *chars, int *out_passes, int *sizes,
                          int *elems) {
    clear_error();
    ProjPlan P;
    if (!plan_host(N, G, perm, chars, P)) return -1;
    if (out_passes) *out_passes = P.passes;
    if (sizes)
        for (int k = 0; k < P.passes; k++) sizes[k] = P.size[k];
    if (elems) std::copy(P.elems.begin(), P.elems.end(), elems);
    return 0;
}

void nqs_kagome_p6m_project_inplace(double *psi, int N, int G, const int *perm, const double *chars) {
    clear_error();
    if (!psi || N <= 0 || N > ED_MAX_N || G <= 0 || !perm || !chars) {
        set_error("invalid projector arguments");
        return;
    }
    if (!ensure_context()) return;
    ProjPlan *P = plan_get(N, G, perm, chars);
    if (!P) return;
    const unsigned dim = 1u << N;
    cudaStream_t st = ctx().stream;
    DevBuf<double> a, t;
    if (!a.ensure(dim) || !t.ensure(dim)) return;
    double *pa = a.p, *pt = t.p;
    if (!NQS_CUDA(cudaMemcpyAsync(pa, psi, sizeof(double) * dim, cudaMemcpyHostToDevice, st)) ||
        !project(*P, pa, pt, dim, nullptr, st))
        return;
    if (NQS_CUDA(cudaMemcpyAsync(psi, pa, sizeof(double) * dim, cudaMemcpyDeviceToHost, st)))
        NQS_CUDA(cudaStreamSynchronize(st));
}

}  // extern "C"
