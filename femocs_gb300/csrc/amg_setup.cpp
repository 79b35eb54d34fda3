// Host construction of the multigrid hierarchy (see amg.h).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>

#include "amg.h"
#include "prepared.h"

#include <cstdio>
#include <cstdlib>

namespace fgb {

namespace {

// read-only view of a CSR matrix (the level-0 system is used in place, not copied)
struct CsrRef {
    int n_rows, n_cols;
    const int64_t* ptr;
    const int32_t* col;
    const double* val;
};
CsrRef ref(const CsrD& M) { return {M.n_rows, M.n_cols, M.ptr.data(), M.col.data(), M.val.data()}; }

CsrD transpose(const CsrD& P) {
    CsrD R;
    R.n_rows = P.n_cols;
    R.n_cols = P.n_rows;
    R.ptr.assign(R.n_rows + 1, 0);
    for (int32_t c : P.col) R.ptr[c + 1]++;
    for (int i = 0; i < R.n_rows; ++i) R.ptr[i + 1] += R.ptr[i];
    R.col.resize(P.nnz());
    R.val.resize(P.nnz());
    std::vector<int64_t> pos(R.ptr.begin(), R.ptr.end() - 1);
    for (int i = 0; i < P.n_rows; ++i)
        for (int64_t k = P.ptr[i]; k < P.ptr[i + 1]; ++k) {
            const int64_t q = pos[P.col[k]]++;
            R.col[q] = i;
            R.val[q] = P.val[k];
        }
    return R;
}

// Rows of a sparse product assembled with a dense accumulator per thread. `row_terms(i, f)`
// calls f(col, value) for every term of output row i.
template <typename RowTerms>
CsrD accumulate_rows(int n_rows, int n_cols, RowTerms row_terms) {
    std::vector<std::vector<std::pair<int32_t, double>>> rows(n_rows);
#pragma omp parallel
    {
        std::vector<double> acc(n_cols, 0.0);
        std::vector<int32_t> mark(n_cols, -1), list;
        list.reserve(1024);
        // small chunks: the coarse levels have few rows, each with hundreds of terms
#pragma omp for schedule(dynamic, 8)
        for (int i = 0; i < n_rows; ++i) {
            list.clear();
            row_terms(i, [&](int32_t c, double v) {
                if (mark[c] != i) {
                    mark[c] = i;
                    acc[c] = 0.0;
                    list.push_back(c);
                }
                acc[c] += v;
            });
            std::sort(list.begin(), list.end());
            auto& out = rows[i];
            out.reserve(list.size());
            for (int32_t c : list) out.push_back({c, acc[c]});
        }
    }
    CsrD C;
    C.n_rows = n_rows;
    C.n_cols = n_cols;
    C.ptr.assign(n_rows + 1, 0);
    for (int i = 0; i < n_rows; ++i) C.ptr[i + 1] = C.ptr[i] + (int64_t)rows[i].size();
    C.col.resize(C.ptr[n_rows]);
    C.val.resize(C.ptr[n_rows]);
    for (int i = 0; i < n_rows; ++i) {
        int64_t q = C.ptr[i];
        for (auto& e : rows[i]) {
            C.col[q] = e.first;
            C.val[q] = e.second;
            ++q;
        }
    }
    return C;
}

// C = A B, row by row
CsrD spgemm(const CsrRef& A, const CsrD& B) {
    return accumulate_rows(A.n_rows, B.n_cols, [&](int i, auto&& add) {
        for (int64_t a = A.ptr[i]; a < A.ptr[i + 1]; ++a) {
            const int j = A.col[a];
            const double w = A.val[a];
            for (int64_t b = B.ptr[j]; b < B.ptr[j + 1]; ++b) add(B.col[b], w * B.val[b]);
        }
    });
}

// Galerkin operator R A P. With a very sparse P (the geometric level: at most 4 entries
// per row) one triple loop per coarse row is cheapest; the smoothed prolongations are
// denser, and R (A P) keeps the cost linear in the fill of A P.
CsrD rap(const CsrD& R, const CsrRef& A, const CsrD& P) {
    if (P.nnz() <= 4 * (int64_t)P.n_rows)
        return accumulate_rows(R.n_rows, P.n_cols, [&](int I, auto&& add) {
            for (int64_t a = R.ptr[I]; a < R.ptr[I + 1]; ++a) {
                const int i = R.col[a];
                const double ri = R.val[a];
                for (int64_t b = A.ptr[i]; b < A.ptr[i + 1]; ++b) {
                    const int j = A.col[b];
                    const double w = ri * A.val[b];
                    for (int64_t c = P.ptr[j]; c < P.ptr[j + 1]; ++c) add(P.col[c], w * P.val[c]);
                }
            }
        });
    return spgemm(ref(R), spgemm(A, P));
}

std::vector<double> diag_of(const CsrRef& A) {
    std::vector<double> d(A.n_rows, 1.0);
    for (int i = 0; i < A.n_rows; ++i)
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (A.col[k] == i) d[i] = A.val[k];
    return d;
}

// largest eigenvalue of D^-1 A by power iteration from a fixed pseudo-random start
double lambda_max(const CsrRef& A, int iters = 15) {
    const int n = A.n_rows;
    std::vector<double> d = diag_of(A), x(n), y(n);
    uint64_t s = 0x12345678abcdefull;
    for (int i = 0; i < n; ++i) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        x[i] = (double)((s >> 11) & 0xfffff) / 1048576.0 - 0.5;
    }
    double lam = 1.0;
    // ||y||^2 from partial sums over fixed chunks of rows, added in chunk order: the same
    // value at any thread count and schedule
    constexpr int kChunk = 256;  // coarse levels have a few thousand dense-ish rows
    const int nch = (n + kChunk - 1) / kChunk;
    std::vector<double> part(nch);
    for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
        for (int ch = 0; ch < nch; ++ch) {
            double sq = 0.0;
            for (int i = ch * kChunk; i < std::min(n, (ch + 1) * kChunk); ++i) {
                double acc = 0.0;
                for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) acc += A.val[k] * x[A.col[k]];
                y[i] = acc / d[i];
                sq += y[i] * y[i];
            }
            part[ch] = sq;
        }
        double nrm = 0.0;
        for (int ch = 0; ch < nch; ++ch) nrm += part[ch];
        nrm = std::sqrt(nrm);
        if (nrm == 0) return 1.0;
        double xn = 0.0;
        for (int i = 0; i < n; ++i) xn += x[i] * x[i];
        lam = nrm / std::sqrt(xn);
        for (int i = 0; i < n; ++i) x[i] = y[i] / nrm;
    }
    return lam;
}

// Greedy aggregation on the strong-connection graph (|a_ij| >= theta sqrt(a_ii a_jj)):
// roots with no aggregated strong neighbour take their whole neighbourhood, the remaining
// nodes join the aggregate they are most strongly connected to, leftovers stay alone.
int aggregate(const CsrD& A, double theta, std::vector<int32_t>& agg) {
    const int n = A.n_rows;
    std::vector<double> d = diag_of(ref(A));
    auto strong = [&](int i, int64_t k) {
        const int j = A.col[k];
        return j != i && A.val[k] != 0.0 && std::fabs(A.val[k]) >= theta * std::sqrt(std::fabs(d[i] * d[j]));
    };
    agg.assign(n, -1);
    int na = 0;
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free_nb = true;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1] && free_nb; ++k)
            if (strong(i, k) && agg[A.col[k]] >= 0) free_nb = false;
        if (!free_nb) continue;
        agg[i] = na;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (strong(i, k)) agg[A.col[k]] = na;
        ++na;
    }
    std::vector<int32_t> first(agg);
    for (int i = 0; i < n; ++i) {
        if (first[i] >= 0) continue;
        double best = -1.0;
        int32_t ba = -1;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (strong(i, k) && first[A.col[k]] >= 0 && std::fabs(A.val[k]) > best) {
                best = std::fabs(A.val[k]);
                ba = first[A.col[k]];
            }
        agg[i] = ba;
    }
    for (int i = 0; i < n; ++i)
        if (agg[i] < 0) agg[i] = na++;
    return na;
}

// Inverse of a dense SPD matrix (row major, n up to a few thousand): Cholesky A = L L^T,
// X = L^-1 by forward substitution one column at a time (columns in parallel), then
// A^-1 = X^T X. X is kept transposed (Xt row c = column c of X) so that every inner loop
// runs over contiguous memory.
std::vector<double> spd_inverse(const std::vector<double>& A, int n) {
    std::vector<double> L(A);
    for (int j = 0; j < n; ++j) {
        const double* lj = &L[(size_t)j * n];
        double s = lj[j];
        for (int k = 0; k < j; ++k) s -= lj[k] * lj[k];
        FGB_REQUIRE(s > 0, "coarsest multigrid operator is not positive definite");
        const double ljj = std::sqrt(s);
        L[(size_t)j * n + j] = ljj;
#pragma omp parallel for schedule(static)
        for (int i = j + 1; i < n; ++i) {
            double* li = &L[(size_t)i * n];
            double t = li[j];
            for (int k = 0; k < j; ++k) t -= li[k] * lj[k];
            li[j] = t / ljj;
        }
    }
    std::vector<double> Xt((size_t)n * n, 0.0);
#pragma omp parallel for schedule(dynamic, 8)
    for (int c = 0; c < n; ++c) {
        double* x = &Xt[(size_t)c * n];
        for (int i = c; i < n; ++i) {
            const double* li = &L[(size_t)i * n];
            double t = i == c ? 1.0 : 0.0;
            for (int k = c; k < i; ++k) t -= li[k] * x[k];
            x[i] = t / li[i];
        }
    }
    std::vector<double> inv((size_t)n * n, 0.0);
#pragma omp parallel for schedule(dynamic, 8)
    for (int a = 0; a < n; ++a) {
        const double* xa = &Xt[(size_t)a * n];
        for (int b = a; b < n; ++b) {
            const double* xb = &Xt[(size_t)b * n];
            double t = 0.0;
            for (int k = b; k < n; ++k) t += xa[k] * xb[k];
            inv[(size_t)a * n + b] = t;
            inv[(size_t)b * n + a] = t;
        }
    }
    return inv;
}

}  // namespace

AmgHost build_amg(const PreparedMesh& pm, const FemStructure& fs, const std::vector<double>& a0_val,
                  const std::vector<int8_t>& fixed, const AmgOptions& opt) {
    const auto t0 = std::chrono::steady_clock::now();
    // FGB_AMG_VERBOSE=1 prints the setup phases to stderr
    const bool verbose = std::getenv("FGB_AMG_VERBOSE") != nullptr;
    auto tlast = t0;
    auto phase = [&](const char* what, long long rows) {
        const auto t = std::chrono::steady_clock::now();
        if (verbose)
            std::fprintf(stderr, "amg setup: %-28s rows %9lld  %9.1f ms\n", what, rows,
                         std::chrono::duration<double, std::milli>(t - tlast).count());
        tlast = t;
    };
    AmgHost h;
    const int n0 = fs.n_dofs;
    // ---- level 0: the assembled system after Dirichlet elimination
    AmgHostLevel l0;
    l0.A.n_rows = l0.A.n_cols = n0;
    l0.A.ptr = fs.rowptr;  // structure only; the values stay in the caller's array
    const CsrRef A0{n0, n0, fs.rowptr.data(), fs.col.data(), a0_val.data()};
    FGB_REQUIRE((int64_t)a0_val.size() == fs.nnz(), "level-0 values do not match the sparsity pattern");

    // ---- geometric first coarsening: free dofs on tet vertices, P1 interpolation weights
    std::vector<int32_t> cidx(n0, -1);
    int n1 = 0;
    for (int d = 0; d < n0; ++d) {
        const int node = fs.dof2node[d];
        if (node < pm.hex.n_tetnodes && !fixed[d]) cidx[d] = n1++;
    }
    FGB_REQUIRE(n1 > 0, "no free tet vertex for the coarse level");
    CsrD P0;
    P0.n_rows = n0;
    P0.n_cols = n1;
    P0.ptr.assign(n0 + 1, 0);
    for (int d = 0; d < n0; ++d) {
        if (!fixed[d]) {
            const int32_t* par = &pm.hex.parents[4 * (size_t)fs.dof2node[d]];
            int k = 0;
            while (k < 4 && par[k] >= 0) ++k;
            for (int q = 0; q < k; ++q) {
                const int dq = fs.node2dof[par[q]];
                if (dq >= 0 && cidx[dq] >= 0) {
                    P0.col.push_back(cidx[dq]);
                    P0.val.push_back(1.0 / k);
                }
            }
        }
        P0.ptr[d + 1] = (int64_t)P0.col.size();
    }
    l0.P = P0;
    l0.R = transpose(P0);
    phase("geometric prolongation", n1);
    l0.lambda = opt.level0_lambda > 0 ? opt.level0_lambda : lambda_max(A0);
    phase("lambda_max level 0", n0);
    CsrD A1 = rap(l0.R, A0, l0.P);
    phase("Galerkin product level 1", n1);
    h.levels.push_back(std::move(l0));

    // ---- smoothed aggregation below
    CsrD A = std::move(A1);
    while (A.n_rows > opt.max_coarse && (int)h.levels.size() < opt.max_levels - 1) {
        AmgHostLevel lv;
        lv.lambda = lambda_max(ref(A));
        std::vector<int32_t> agg;
        // weak coupling leaves many singletons: lower the strength threshold until the level
        // coarsens by at least 2, ending with every nonzero coupling counted as strong
        int na = aggregate(A, opt.strength, agg);
        for (double th = opt.strength / 4; na > A.n_rows / 2 && th > 1e-4; th /= 4) na = aggregate(A, th, agg);
        if (na > A.n_rows / 2) na = aggregate(A, 0.0, agg);
        phase("lambda_max + aggregation", A.n_rows);
        if (na >= A.n_rows * 0.8) break;  // no useful coarsening left
        std::vector<double> dA = diag_of(ref(A));
        const double omega = 4.0 / (3.0 * lv.lambda);
        // P = (I - omega D^-1 A) P_tent, P_tent[i][agg(i)] = 1
        CsrD P = accumulate_rows(A.n_rows, na, [&](int i, auto&& add) {
            add(agg[i], 1.0);
            const double s = -omega / dA[i];
            for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) add(agg[A.col[k]], s * A.val[k]);
        });
        CsrD R = transpose(P);
        CsrD Ac = rap(R, ref(A), P);
        phase("smoothed prolongation + RAP", na);
        lv.A = std::move(A);
        lv.P = std::move(P);
        lv.R = std::move(R);
        h.levels.push_back(std::move(lv));
        A = std::move(Ac);
    }
    // ---- coarsest: dense inverse
    FGB_REQUIRE(A.n_rows <= opt.max_dense, "multigrid coarsening stalled at " + std::to_string(A.n_rows) +
                                               " rows, above the dense coarsest-level limit");
    AmgHostLevel last;
    last.lambda = lambda_max(ref(A));
    const int nc = A.n_rows;
    std::vector<double> dense((size_t)nc * nc, 0.0);
    for (int i = 0; i < nc; ++i)
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) dense[(size_t)i * nc + A.col[k]] = A.val[k];
    h.coarse_inv = spd_inverse(dense, nc);
    h.n_coarse = nc;
    phase("dense inverse", nc);
    last.A = std::move(A);
    h.levels.push_back(std::move(last));
    h.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return h;
}

}  // namespace fgb
