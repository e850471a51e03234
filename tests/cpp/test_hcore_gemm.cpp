// C++ check of the HCore++-shaped adapter (include/hcorepp_gb300/hcore.hpp), modelled on the
// reference's integration test tests/api/AdvancedGemmTest.cpp: every tile combination with
// alpha = 3.5, beta = 2.5, compressed operands built by CompressedTile(dense, params), and the
// reference's pass rule (AdvancedGemmTest.cpp:245-256):
//   ||C_ref - C||_inf / (sqrt(k + 2) |alpha| ||A||_inf ||B||_inf + 2 |beta| ||C||_inf) < 3 * accuracy.
// Inputs: Q1 diag(10^-i) Q2^T with seeded random orthogonal Q1, Q2 -- the singular values the
// reference's generate_dense_matrix asks dlatms for (src/helpers/MatrixHelpers.cpp:22-31); the
// LAPACK generator itself is not linked here.  Exit status 0 = every case passed.
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
    return failures == 0 ? 0 : 1;
}
