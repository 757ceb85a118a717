// Ruge-Stueben setup of the AMG preconditioner, on the host.
//
// The hierarchy is defined by a greedy, sequential C/F selection
// (AMGPreconditioner::coarsen, src/solver/AMGPreconditioner.cpp:69-113): a
// parallel coarsening would pick other C points and change every operator
// below the fine level, so the setup stays the reference's algorithm, and
// only the V-cycle, which the Krylov iteration applies every step, runs on the
// device (amg.cu).  The selection here is the same one done in
// O(nnz log n) instead of the reference's O(n^2) rescans: the undecided point
// with the largest lambda, the smallest index on ties, comes off a max-heap
// whose stale entries (points decided since, or whose lambda has grown) are
// skipped.  Lambdas only grow while a point is undecided, so the top live
// entry is always the reference's choice.
//
// Every floating-point operation is the reference's, in its order (this file
// is compiled with -ffp-contract=off): the interpolation weights -a_ij * (1 /
// a_ii), each Galerkin row summed in the order its products are met with its
// columns sorted afterwards, the dense LU with partial pivoting.
#include "amg.hpp"
#include "simall_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <queue>

namespace simall {

namespace {

double diag_of(const AmgCsr &A, int32_t i)
{
    for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k)
        if (A.ci[k] == i)
            return A.v[k];
    return 0.0;
}

// build_strong (:43-67): j is a strong coupling of i when -a_ij >= theta
// max_k(-a_ik), k != i; rows without a negative coupling have none.
void strong(const AmgCsr &A, double theta, std::vector<int32_t> &sp, std::vector<int32_t> &sj)
{
    const int32_t n = A.n;
    sp.assign(static_cast<size_t>(n) + 1, 0);
    sj.clear();
    sj.reserve(A.ci.size());
    for (int32_t i = 0; i < n; ++i) {
        double maxOff = 0.0;
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            if (A.ci[k] == i)
                continue;
            const double m = -A.v[k];
            maxOff = (maxOff < m) ? m : maxOff;  // std::max
        }
        if (maxOff > 0.0) {
            const double thr = theta * maxOff;
            for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
                if (A.ci[k] == i)
                    continue;
                if (-A.v[k] >= thr)
                    sj.push_back(A.ci[k]);
            }
        }
        sp[i + 1] = static_cast<int32_t>(sj.size());
    }
}

// coarsen (:69-113); cf[i] = 1 C point, 0 F point.  Returns the C count.
int32_t coarsen(int32_t n, const std::vector<int32_t> &sp, const std::vector<int32_t> &sj, std::vector<int32_t> &cf)
{
    std::vector<int32_t> tp(static_cast<size_t>(n) + 1, 0), tj(sj.size());
    for (int32_t j : sj)
        ++tp[j + 1];
    for (int32_t i = 0; i < n; ++i)
        tp[i + 1] += tp[i];
    {
        std::vector<int32_t> fill(tp.begin(), tp.end() - 1);
        for (int32_t i = 0; i < n; ++i)
            for (int32_t q = sp[i]; q < sp[i + 1]; ++q)
                tj[fill[sj[q]]++] = i;  // S^T rows in ascending i
    }
    std::vector<int32_t> lambda(n);
    cf.assign(n, -1);
    // key: lambda in the high word, then the complement of the index, so the
    // largest key is the largest lambda with the smallest index
    auto key = [](int32_t lam, int32_t i) {
        return (static_cast<uint64_t>(static_cast<uint32_t>(lam)) << 32) | (0xffffffffu - static_cast<uint32_t>(i));
    };
    std::priority_queue<uint64_t> heap;
    {
        std::vector<uint64_t> init(n);
        for (int32_t i = 0; i < n; ++i) {
            lambda[i] = tp[i + 1] - tp[i];
            init[i] = key(lambda[i], i);
        }
        heap = std::priority_queue<uint64_t>(std::less<uint64_t>(), std::move(init));
    }
    while (!heap.empty()) {
        const uint64_t top = heap.top();
        heap.pop();
        const int32_t best = static_cast<int32_t>(0xffffffffu - static_cast<uint32_t>(top & 0xffffffffu));
        const int32_t lam = static_cast<int32_t>(top >> 32);
        if (cf[best] >= 0 || lambda[best] != lam)
            continue;  // stale
        cf[best] = 1;
        for (int32_t q = tp[best]; q < tp[best + 1]; ++q) {
            const int32_t j = tj[q];
            if (cf[j] < 0) {
                cf[j] = 0;
                for (int32_t r = sp[j]; r < sp[j + 1]; ++r) {
                    const int32_t k = sj[r];
                    if (cf[k] < 0) {
                        ++lambda[k];
                        heap.push(key(lambda[k], k));
                    }
                }
            }
        }
        lambda[best] = -1;
    }
    int32_t nc = 0;
    for (int32_t i = 0; i < n; ++i) {
        if (cf[i] < 0)
            cf[i] = 1;
        nc += cf[i] == 1 ? 1 : 0;
    }
    return nc;
}

// build_prolongation (:115-151): C rows copy their coarse value, F rows
// interpolate from their C neighbours with -a_ij / a_ii.
void prolongation(const AmgCsr &A, const std::vector<int32_t> &cf, AmgCsr &P)
{
    const int32_t nf = A.n;
    std::vector<int32_t> cid(nf, -1);
    int32_t nc = 0;
    for (int32_t i = 0; i < nf; ++i)
        if (cf[i] == 1)
            cid[i] = nc++;
    P.n = nf;
    P.rp.assign(static_cast<size_t>(nf) + 1, 0);
    P.ci.clear();
    P.v.clear();
    for (int32_t i = 0; i < nf; ++i) {
        if (cf[i] == 1) {
            P.ci.push_back(cid[i]);
            P.v.push_back(1.0);
        } else {
            const double dii = diag_of(A, i);
            const double inv = (std::fabs(dii) > 1e-30) ? 1.0 / dii : 0.0;
            for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
                const int32_t j = A.ci[k];
                if (j == i || cf[j] != 1)
                    continue;
                P.ci.push_back(cid[j]);
                P.v.push_back(-A.v[k] * inv);
            }
        }
        P.rp[i + 1] = static_cast<int32_t>(P.ci.size());
    }
}

// transpose (:153-174): row c of T lists the rows i of M in ascending order.
void transpose(const AmgCsr &M, int32_t newRows, AmgCsr &T)
{
    T.n = newRows;
    T.rp.assign(static_cast<size_t>(newRows) + 1, 0);
    for (int32_t c : M.ci)
        ++T.rp[c + 1];
    for (int32_t i = 0; i < newRows; ++i)
        T.rp[i + 1] += T.rp[i];
    T.ci.assign(M.ci.size(), 0);
    T.v.assign(M.v.size(), 0.0);
    std::vector<int32_t> cur(newRows, 0);
    for (int32_t i = 0; i < M.n; ++i)
        for (int32_t k = M.rp[i]; k < M.rp[i + 1]; ++k) {
            const int32_t c = M.ci[k];
            const int32_t dst = T.rp[c] + cur[c]++;
            T.ci[dst] = i;
            T.v[dst] = M.v[k];
        }
}

// C = L * M as triple_product_RAP forms each of its two products (:176-246).
void multiply(const AmgCsr &L, const AmgCsr &M, int32_t ncols, AmgCsr &C)
{
    std::vector<double> acc(ncols, 0.0);
    std::vector<int32_t> mark(ncols, -1), cols;
    C.n = L.n;
    C.rp.assign(static_cast<size_t>(L.n) + 1, 0);
    C.ci.clear();
    C.v.clear();
    for (int32_t i = 0; i < L.n; ++i) {
        cols.clear();
        for (int32_t k = L.rp[i]; k < L.rp[i + 1]; ++k) {
            const int32_t j = L.ci[k];
            const double lij = L.v[k];
            for (int32_t kp = M.rp[j]; kp < M.rp[j + 1]; ++kp) {
                const int32_t c = M.ci[kp];
                const double v = lij * M.v[kp];
                if (mark[c] != i) {
                    mark[c] = i;
                    acc[c] = v;
                    cols.push_back(c);
                } else {
                    acc[c] += v;
                }
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int32_t c : cols) {
            C.ci.push_back(c);
            C.v.push_back(acc[c]);
        }
        C.rp[i + 1] = static_cast<int32_t>(C.ci.size());
    }
}

}  // namespace

void amg_build_hierarchy(int32_t n, const int32_t *rp, const int32_t *ci, const double *v, const AmgParams &prm,
                         AmgHierarchy &h)
{
    h.A.clear();
    h.P.clear();
    h.R.clear();
    AmgCsr top;
    top.n = n;
    top.rp.assign(rp, rp + n + 1);
    top.ci.assign(ci, ci + rp[n]);
    top.v.assign(v, v + rp[n]);
    h.A.push_back(std::move(top));
    for (int lvl = 0; lvl < prm.maxLevels - 1; ++lvl) {
        const AmgCsr &Af = h.A.back();
        const int32_t nf = Af.n;
        if (nf <= prm.coarseThreshold)
            break;
        std::vector<int32_t> sp, sj, cf;
        strong(Af, prm.theta, sp, sj);
        const int32_t nc = coarsen(nf, sp, sj, cf);
        if (nc == 0 || nc >= nf)
            break;
        AmgCsr P, R, AP, Ac;
        prolongation(Af, cf, P);
        transpose(P, nc, R);
        int32_t ncols = 0;
        for (int32_t c : P.ci)
            ncols = std::max(ncols, c + 1);
        multiply(Af, P, ncols, AP);
        multiply(R, AP, ncols, Ac);
        h.P.push_back(std::move(P));
        h.R.push_back(std::move(R));
        h.A.push_back(std::move(Ac));
    }
    // dense LU with partial pivoting of the coarsest operator (:296-322)
    const AmgCsr &Ac = h.A.back();
    const int32_t cn = Ac.n;
    h.coarseN = cn;
    h.lu.assign(static_cast<size_t>(cn) * cn, 0.0);
    double *LU = h.lu.data();
    for (int32_t i = 0; i < cn; ++i)
        for (int32_t k = Ac.rp[i]; k < Ac.rp[i + 1]; ++k)
            LU[static_cast<size_t>(i) * cn + Ac.ci[k]] = Ac.v[k];
    for (int32_t k = 0; k < cn; ++k) {
        int32_t piv = k;
        double pivVal = std::fabs(LU[static_cast<size_t>(k) * cn + k]);
        for (int32_t i = k + 1; i < cn; ++i) {
            const double a = std::fabs(LU[static_cast<size_t>(i) * cn + k]);
            if (a > pivVal) {
                pivVal = a;
                piv = i;
            }
        }
        if (pivVal < 1e-30)
            continue;
        if (piv != k)
            for (int32_t j = 0; j < cn; ++j)
                std::swap(LU[static_cast<size_t>(k) * cn + j], LU[static_cast<size_t>(piv) * cn + j]);
        const double dinv = 1.0 / LU[static_cast<size_t>(k) * cn + k];
        for (int32_t i = k + 1; i < cn; ++i) {
            const double f = LU[static_cast<size_t>(i) * cn + k] * dinv;
            LU[static_cast<size_t>(i) * cn + k] = f;
            for (int32_t j = k + 1; j < cn; ++j)
                LU[static_cast<size_t>(i) * cn + j] -= f * LU[static_cast<size_t>(k) * cn + j];
        }
    }
}

}  // namespace simall

namespace {

// FNV-1a over 64-bit words: the digest both this library and the oracle take
// of a hierarchy.
struct Digest {
    uint64_t h = 0xcbf29ce484222325ULL;
    void word(uint64_t w)
    {
        h ^= w;
        h *= 0x100000001b3ULL;
    }
    void ints(const std::vector<int32_t> &a)
    {
        for (int32_t v : a)
            word(static_cast<uint64_t>(static_cast<uint32_t>(v)));
    }
    void reals(const std::vector<double> &a)
    {
        for (double v : a) {
            uint64_t w;
            std::memcpy(&w, &v, sizeof w);
            word(w);
        }
    }
    void csr(const simall::AmgCsr &m)
    {
        ints(m.rp);
        ints(m.ci);
        reals(m.v);
    }
};

}  // namespace

extern "C" int simall_amg_hierarchy_digest(int64_t n, const int32_t *rowPtr, const int32_t *colIdx,
                                           const double *values, int *nlev, int32_t *rows, int max_levels,
                                           uint64_t *digest)
{
    if (n <= 0 || n > INT32_MAX - 1 || !rowPtr || !colIdx || !values || !nlev || !digest ||
        (max_levels > 0 && !rows))
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall::AmgHierarchy h;
    simall::amg_build_hierarchy(static_cast<int32_t>(n), rowPtr, colIdx, values, simall::AmgParams{}, h);
    Digest d;
    for (size_t l = 0; l < h.A.size(); ++l) {
        d.csr(h.A[l]);
        if (l < h.P.size()) {
            d.csr(h.P[l]);
            d.csr(h.R[l]);
        }
    }
    d.reals(h.lu);
    *nlev = static_cast<int>(h.A.size());
    for (int l = 0; l < *nlev && l < max_levels; ++l)
        rows[l] = h.A[l].n;
    *digest = d.h;
    return SIMALL_OK;
}
