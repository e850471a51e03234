// C++ check of the HCore++-shaped adapter (include/hcorepp_gb300/hcore.hpp), modelled on the
// reference's integration test tests/api/AdvancedGemmTest.cpp: every tile combination with
// alpha = 3.5, beta = 2.5, compressed operands built by CompressedTile(dense, params), and the
// reference's pass rule (AdvancedGemmTest.cpp:245-256):
//   ||C_ref - C||_inf / (sqrt(k + 2) |alpha| ||A||_inf ||B||_inf + 2 |beta| ||C||_inf) < 3 * accuracy.
// Inputs: Q1 diag(10^-i) Q2^T with seeded random orthogonal Q1, Q2 -- the singular values the
// reference's generate_dense_matrix asks dlatms for (src/helpers/MatrixHelpers.cpp:22-31); the
// LAPACK generator itself is not linked here.  Then the Cholesky-flow operations (Potrf, Trsm, Syrk,
// Gemm with aCholesky = true) against host loops, and a TilePacker round trip.  Exit status 0 =
// every case passed.
#include <hcorepp_gb300/hcore.hpp>

#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

using namespace hcorepp;
using M = std::vector<double>;

static M random_orthogonal(int n, std::mt19937_64 &g) {
    std::normal_distribution<double> nd(0.0, 1.0);
    M q((size_t) n * n);
    for (auto &v : q) v = nd(g);
    for (int j = 0; j < n; j++) {  // modified Gram-Schmidt, twice for orthogonality to rounding
        for (int pass = 0; pass < 2; pass++)
            for (int k = 0; k < j; k++) {
                double d = 0;
                for (int i = 0; i < n; i++) d += q[i + (size_t) k * n] * q[i + (size_t) j * n];
                for (int i = 0; i < n; i++) q[i + (size_t) j * n] -= d * q[i + (size_t) k * n];
            }
        double s = 0;
        for (int i = 0; i < n; i++) s += q[i + (size_t) j * n] * q[i + (size_t) j * n];
        s = 1.0 / std::sqrt(s);
        for (int i = 0; i < n; i++) q[i + (size_t) j * n] *= s;
    }
    return q;
}

static M graded_matrix(int n, unsigned seed) {
    std::mt19937_64 g(seed);
    M q1 = random_orthogonal(n, g), q2 = random_orthogonal(n, g), a((size_t) n * n, 0.0);
    const int r = std::min(n, 20);  // 10^-i below 1e-20 is far under any accuracy tested
    for (int l = 0; l < r; l++) {
        const double s = std::pow(10.0, -l);
        for (int j = 0; j < n; j++) {
            const double b = s * q2[j + (size_t) l * n];
            for (int i = 0; i < n; i++) a[i + (size_t) j * n] += q1[i + (size_t) l * n] * b;
        }
    }
    return a;
}

static double norm_inf(const M &a, int m, int n) {
    double best = 0;
    for (int i = 0; i < m; i++) {
        double s = 0;
        for (int j = 0; j < n; j++) s += std::fabs(a[i + (size_t) j * m]);
        best = std::max(best, s);
    }
    return best;
}

static M to_host_dense(const operators::Tile<double> &t) {
    const int m = (int) t.GetNumOfRows(), n = (int) t.GetNumOfCols();
    M out((size_t) m * n, 0.0);
    if (t.isDense()) {
        auto &d = static_cast<const operators::DenseTile<double> &>(t);
        cudaMemcpy(out.data(), d.GetTileSubMatrix(0), sizeof(double) * out.size(), cudaMemcpyDeviceToHost);
        return out;
    }
    auto &c = static_cast<const operators::CompressedTile<double> &>(t);
    const int r = (int) c.GetTileRank();
    M u((size_t) m * r), v((size_t) r * n);
    cudaMemcpy(u.data(), c.GetUMatrix(), sizeof(double) * u.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(v.data(), c.GetVMatrix(), sizeof(double) * v.size(), cudaMemcpyDeviceToHost);
    for (int j = 0; j < n; j++)
        for (int l = 0; l < r; l++) {
            const double vl = v[l + (size_t) j * r];
            for (int i = 0; i < m; i++) out[i + (size_t) j * m] += u[i + (size_t) l * m] * vl;
        }
    return out;
}

// A compressed tile as the Cholesky routines read it: U (m x r) times W^T, W = V region (n x r, ld n).
static M vt_dense(const operators::CompressedTile<double> &c) {
    const int m = (int) c.GetNumOfRows(), n = (int) c.GetNumOfCols(), r = (int) c.GetTileRank();
    M u((size_t) m * r), w((size_t) n * r), out((size_t) m * n, 0.0);
    cudaMemcpy(u.data(), c.GetUMatrix(), sizeof(double) * u.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(w.data(), c.GetVMatrix(), sizeof(double) * w.size(), cudaMemcpyDeviceToHost);
    for (int j = 0; j < n; j++)
        for (int l = 0; l < r; l++) {
            const double wl = w[j + (size_t) l * n];
            for (int i = 0; i < m; i++) out[i + (size_t) j * m] += u[i + (size_t) l * m] * wl;
        }
    return out;
}

static M host_of(const double *dev, size_t count) {
    M h(count);
    cudaMemcpy(h.data(), dev, sizeof(double) * count, cudaMemcpyDeviceToHost);
    return h;
}

static bool report(const char *name, int n, double err, double tol) {
    const bool pass = err < tol;
    std::printf("|%-5s|%-5d|%-14.3e|%-5s|%-6s|\n", name, n, err, "-", pass ? "Pass" : "Fail");
    return pass;
}

// Potrf, Trsm, Syrk and Gemm(aCholesky = true) of the Cholesky flow (HCore.cpp:23-344, :482-647).
static int cholesky_ops(kernels::RunContext &ctx, dataunits::MemoryUnit<double> &mem) {
    const int n = 96;
    int failures = 0;
    size_t flops = 0;
    std::mt19937_64 g(5);
    M q = random_orthogonal(n, g), spd((size_t) n * n, 0.0);
    for (int l = 0; l < n; l++)
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++) spd[i + (size_t) j * n] += q[i + (size_t) l * n] * (1.0 + l) * q[j + (size_t) l * n];
    operators::DenseTile<double> L(n, n, spd.data(), n, ctx);
    api::HCore<double>::Potrf(L, blas::Uplo::Lower, ctx, flops, mem);
    ctx.Sync();
    M lh = host_of(L.GetTileSubMatrix(0), (size_t) n * n);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < j; i++) lh[i + (size_t) j * n] = 0.0;
    double e = 0, s = 0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double t = 0;
            for (int l = 0; l < n; l++) t += lh[i + (size_t) l * n] * lh[j + (size_t) l * n];
            e = std::max(e, std::fabs(t - spd[i + (size_t) j * n]));
            s = std::max(s, std::fabs(spd[i + (size_t) j * n]));
        }
    failures += !report("POTRF", n, e / s, 1e-13);

    operators::CompressionParameters params(1e-10);
    M bd = graded_matrix(n, 71), ad = graded_matrix(n, 72), cd = graded_matrix(n, 73);
    operators::CompressedTile<double> B(n, n, bd.data(), n, params, blas::Layout::ColMajor, ctx);
    const int rb = (int) B.GetTileRank();
    M w0 = host_of(B.GetVMatrix(), (size_t) n * rb);
    api::HCore<double>::Trsm(blas::Side::Left, blas::Uplo::Lower, blas::Op::NoTrans, blas::Diag::NonUnit, 1.0, L, B,
                             ctx, flops, mem);
    ctx.Sync();
    M w1 = host_of(B.GetVMatrix(), (size_t) n * rb);
    e = 0, s = 0;
    for (int c = 0; c < rb; c++)
        for (int i = 0; i < n; i++) {
            double t = 0;
            for (int l = 0; l <= i; l++) t += lh[i + (size_t) l * n] * w1[l + (size_t) c * n];
            e = std::max(e, std::fabs(t - w0[i + (size_t) c * n]));
            s = std::max(s, std::fabs(w0[i + (size_t) c * n]));
        }
    failures += !report("TRSM", n, e / s, 1e-12);

    operators::CompressedTile<double> A(n, n, ad.data(), n, params, blas::Layout::ColMajor, ctx);
    M a_vt = vt_dense(A);
    operators::DenseTile<double> Cd(n, n, cd.data(), n, ctx);
    api::HCore<double>::Syrk(-1.0, A, blas::Op::NoTrans, blas::Uplo::Lower, 0.5, Cd, ctx, flops, mem);
    ctx.Sync();
    M ch = host_of(Cd.GetTileSubMatrix(0), (size_t) n * n);
    e = 0, s = 0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double t = 0;
            if (i >= j) {
                t = 0.5 * cd[i + (size_t) j * n];
                for (int l = 0; l < n; l++) t -= a_vt[i + (size_t) l * n] * a_vt[j + (size_t) l * n];
            }
            e = std::max(e, std::fabs(t - ch[i + (size_t) j * n]));
            s = std::max(s, std::fabs(t));
        }
    failures += !report("SYRK", n, e / s, 1e-12);

    operators::CompressedTile<double> Bc(n, n, bd.data(), n, params, blas::Layout::ColMajor, ctx);
    operators::CompressedTile<double> Cc(n, n, cd.data(), n, params, blas::Layout::ColMajor, ctx);
    M b_vt = vt_dense(Bc), c_vt = vt_dense(Cc), ref((size_t) n * n);
    const double alpha = -1.0, beta = 1.0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            double t = beta * c_vt[i + (size_t) j * n];
            for (int l = 0; l < n; l++) t += alpha * a_vt[i + (size_t) l * n] * b_vt[j + (size_t) l * n];
            ref[i + (size_t) j * n] = t;
        }
    api::HCore<double>::Gemm(alpha, A, blas::Op::NoTrans, Bc, blas::Op::Trans, beta, Cc, ctx, flops, mem, params, true);
    ctx.Sync();
    M out = vt_dense(Cc);
    for (size_t q2 = 0; q2 < out.size(); q2++) out[q2] = ref[q2] - out[q2];
    const double denom = std::sqrt((double) n + 2) * norm_inf(a_vt, n, n) * norm_inf(b_vt, n, n) +
                         2 * norm_inf(c_vt, n, n);
    failures += !report("CHOLG", n, norm_inf(out, n, n) / denom, 3 * 1e-10);
    bool threw = false;
    try {
        api::HCore<double>::Gemm(alpha, A, blas::Op::NoTrans, Bc, blas::Op::NoTrans, beta, Cc, ctx, flops, mem, params,
                                 true);
    } catch (const std::invalid_argument &) {
        threw = true;
    }
    failures += !report("CHOLX", n, threw ? 0.0 : 1.0, 0.5);
    return failures;
}

// TilePacker round trip (TestTilePacker.cpp): unpack -> metadata + buffer, pack -> a tile over the
// same buffer; a product through packed tiles equals the product through the originals bitwise.
static int tile_packer(kernels::RunContext &ctx, dataunits::MemoryUnit<double> &mem) {
    const int n = 128;
    int failures = 0;
    operators::CompressionParameters params(1e-8);
    M ad = graded_matrix(n, 81), bd = graded_matrix(n, 82), cd = graded_matrix(n, 83);
    operators::CompressedTile<double> A(n, n, ad.data(), n, params, blas::Layout::ColMajor, ctx);
    operators::DenseTile<double> B(n, n, bd.data(), n, ctx);
    auto ma = operators::TilePacker<double>::UnPackTile(A, ctx);
    auto mb = operators::TilePacker<double>::UnPackTile(B, ctx);
    const bool meta_ok = ma.first->mType == operators::COMPRESSED && ma.first->mNumOfRows == (size_t) n &&
                         ma.first->mMatrixRank == A.GetTileRank() && ma.first->mMaxRank == A.GetMaxRank() &&
                         ma.second == A.GetUMatrix() && mb.first->mType == operators::DENSE &&
                         mb.second == B.GetTileSubMatrix(0);
    std::unique_ptr<operators::Tile<double>> pa(operators::TilePacker<double>::PackTile(*ma.first, ma.second, ctx));
    std::unique_ptr<operators::Tile<double>> pb(operators::TilePacker<double>::PackTile(*mb.first, mb.second, ctx));
    delete ma.first;
    delete mb.first;
    operators::CompressedTile<double> C1(n, n, cd.data(), n, params, blas::Layout::ColMajor, ctx);
    operators::CompressedTile<double> C2(n, n, cd.data(), n, params, blas::Layout::ColMajor, ctx);
    size_t flops = 0;
    api::HCore<double>::Gemm(1.0, A, blas::Op::NoTrans, B, blas::Op::NoTrans, 1.0, C1, ctx, flops, mem, params);
    api::HCore<double>::Gemm(1.0, *pa, blas::Op::NoTrans, *pb, blas::Op::NoTrans, 1.0, C2, ctx, flops, mem, params);
    ctx.Sync();
    M o1 = to_host_dense(C1), o2 = to_host_dense(C2), a1 = to_host_dense(A), a2 = to_host_dense(*pa);
    double diff = 0;
    for (size_t e = 0; e < o1.size(); e++) diff = std::max(diff, std::fabs(o1[e] - o2[e]) + std::fabs(a1[e] - a2[e]));
    failures += !report("PACK", n, meta_ok ? diff : 1.0, 1e-300);
    return failures;
}

// MemoryUnit's pool semantics (pool/MemoryHandler.hpp:22-157): consecutive slices, exhaustion and
// use before Initialize throw, Reset rewinds and zeroes, Free releases.
static int memory_unit(kernels::RunContext &ctx) {
    int fails = 0;
    dataunits::MemoryUnit<double> unit(ctx);
    bool threw = false;
    try {
        (void) unit.RequestAllocation(1);
    } catch (const std::runtime_error &) {
        threw = true;
    }
    fails += !threw;
    unit.Initialize(1000);
    double *a = unit.RequestAllocation(300), *b = unit.RequestAllocation(700);
    fails += (b != a + 300) || unit.GetPoolAvailableSize() != 0 || unit.GetPoolSize() != 1000;
    threw = false;
    try {
        (void) unit.RequestAllocation(1);
    } catch (const std::runtime_error &) {
        threw = true;
    }
    fails += !threw;
    threw = false;
    try {
        unit.Initialize(10);
    } catch (const std::runtime_error &) {
        threw = true;
    }
    fails += !threw;
    std::vector<double> ones(1000, 1.0), back(1000, -1.0);
    cudaMemcpy(a, ones.data(), sizeof(double) * 1000, cudaMemcpyHostToDevice);
    unit.Reset();
    cudaMemcpyAsync(back.data(), unit.GetData(), sizeof(double) * 1000, cudaMemcpyDeviceToHost, ctx.GetStream());
    cudaStreamSynchronize(ctx.GetStream());
    for (double v : back) fails += v != 0.0;
    fails += unit.GetPoolAvailableSize() != 1000 || unit.RequestAllocation(10) != a;
    unit.Free();
    fails += unit.IsInitialized();
    std::printf("MemoryUnit pool: %s\n", fails ? "Fail" : "Pass");
    return fails ? 1 : 0;
}

int main() {
    kernels::RunContext ctx(0);
    dataunits::MemoryUnit<double> mem(ctx);
    const double alpha = 3.5, beta = 2.5, accuracy = 1e-4;
    const char *combos[] = {"DDD", "DDC", "DCD", "DCC", "CDD", "CDC", "CCD", "CCC"};
    int failures = 0;
    std::printf("|%-5s|%-5s|%-14s|%-5s|%-6s|\n", "Gemm", "n", "error", "Crk", "status");
    for (const char *combo : combos) {
        for (int n : {100, 200, 300}) {
            M ad = graded_matrix(n, 11 + n), bd = graded_matrix(n, 23 + n), cd = graded_matrix(n, 37 + n);
            operators::CompressionParameters params(accuracy);
            std::unique_ptr<operators::Tile<double>> A, B, C;
            auto make = [&](char kind, M &d) -> std::unique_ptr<operators::Tile<double>> {
                if (kind == 'D') return std::make_unique<operators::DenseTile<double>>(n, n, d.data(), n, ctx);
                return std::make_unique<operators::CompressedTile<double>>(n, n, d.data(), n, params,
                                                                          blas::Layout::ColMajor, ctx);
            };
            A = make(combo[0], ad);
            B = make(combo[1], bd);
            C = make(combo[2], cd);
            // The reference product uses the operands exactly as the tiles hold them.
            M ah = to_host_dense(*A), bh = to_host_dense(*B), ch = to_host_dense(*C);
            M ref(ch.size());
            for (size_t e = 0; e < ref.size(); e++) ref[e] = beta * ch[e];
            for (int j = 0; j < n; j++)
                for (int l = 0; l < n; l++) {
                    const double b = alpha * bh[l + (size_t) j * n];
                    for (int i = 0; i < n; i++) ref[i + (size_t) j * n] += ah[i + (size_t) l * n] * b;
                }
            size_t flops = 0;
            api::HCore<double>::Gemm(alpha, *A, blas::Op::NoTrans, *B, blas::Op::NoTrans, beta, *C, ctx, flops, mem,
                                     params);
            ctx.Sync();
            M out = to_host_dense(*C);
            for (size_t e = 0; e < out.size(); e++) out[e] = ref[e] - out[e];
            const double denom = std::sqrt((double) n + 2) * std::fabs(alpha) * norm_inf(ah, n, n) * norm_inf(bh, n, n) +
                                 2 * std::fabs(beta) * norm_inf(ch, n, n);
            const double err = norm_inf(out, n, n) / denom;
            const bool pass = err < 3 * accuracy && flops > 0;
            failures += !pass;
            std::printf("|%-5s|%-5d|%-14.3e|%-5zu|%-6s|\n", combo, n, err, C->GetTileRank(), pass ? "Pass" : "Fail");
        }
    }
    failures += cholesky_ops(ctx, mem);
    failures += tile_packer(ctx, mem);
    failures += memory_unit(ctx);
    return failures == 0 ? 0 : 1;
}
