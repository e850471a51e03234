// C entry points over the reference's OWN CPU implementation (HCore++ compiled from its
// sources with the BLAS++/LAPACK++ shim in oracle/shim).  Test infrastructure only: the
// tests use it to pin the numpy oracle, and bench.py times it as the CPU baseline.
//
// Tiles are passed in the reference's own buffer layout:
//   dense      : rows x cols, column-major, ld = rows
//   compressed : [U: rows x max_rank (ld rows) | V: max_rank x cols (ld = rank)]
// which is CompressedTile's DataHolder layout (Compressed.cpp:50-73, :176-185).
// Caller buffers are wrapped without copies through the runtime-transport path
// (TileMetadata + PackTile, Tile.hpp:30-52, Compressed.cpp:781-789).
#include <hcorepp/api/HCore.hpp>
#include <hcorepp/operators/concrete/Compressed.hpp>
#include <hcorepp/operators/concrete/Dense.hpp>
#include <hcorepp/data-units/memory-handlers/MemoryHandler.hpp>
#include <hcorepp/kernels/ContextManager.hpp>
#include <omp.h>
#include <chrono>
#include <cstring>
#include <exception>
#include <memory>
#include <vector>

using namespace hcorepp;
using namespace hcorepp::operators;

namespace {

std::unique_ptr<Tile<double>> wrap_tile(int kind, int rows, int cols, int rank, int max_rank, double *data,
                                        const kernels::RunContext &ctx) {
    if (kind == 0) {
        return std::unique_ptr<Tile<double>>(
                new DenseTile<double>(rows, cols, data, rows, blas::Layout::ColMajor, ctx, false));
    }
    auto *t = new CompressedTile<double>();
    TileMetadata md(rows, cols, rank, max_rank, rows, blas::Layout::ColMajor, COMPRESSED);
    t->PackTile(md, data, ctx);
    return std::unique_ptr<Tile<double>>(t);
}

CompressionParameters make_params(double acc, int truncated, int fixed_rank, int op_type) {
    return CompressionParameters(acc, false, true, truncated != 0, (size_t) fixed_rank,
                                 op_type == 0 ? common::CompressionType::LAPACK_GESVD
                                              : common::CompressionType::LAPACK_GESDD);
}

}  // namespace

extern "C" {

// Use one BLAS thread per caller thread (the reference's drivers parallelise over tiles).
void hcref_set_blas_threads(int n) { HCGB_CAT3(HCGB_F77_PREFIX, openblas_set_num_threads, )(n); }

// CompressedTile(dense, params) (Compressed.cpp:75-146).  uv_out must hold
// rows*maxR + maxR*cols doubles; it receives the tile buffer.  Returns the rank, or -1.
int hcref_compress(int rows, int cols, const double *dense, double acc, int truncated, int fixed_rank,
                   int op_type, double *uv_out, int *max_rank_out) {
    try {
        auto &ctx = kernels::ContextManager::GetInstance().GetContext();
        std::vector<double> copy(dense, dense + (size_t) rows * cols);
        CompressedTile<double> t(rows, cols, copy.data(), rows, make_params(acc, truncated, fixed_rank, op_type),
                                 blas::Layout::ColMajor, ctx);
        size_t max_rank = t.GetTileRank() > 0 ? (size_t) (t.GetVMatrix() - t.GetUMatrix()) / rows : 0;
        size_t rank = t.GetTileRank();
        std::memcpy(uv_out, t.GetUMatrix(), sizeof(double) * rows * rank);
        std::memcpy(uv_out + (size_t) rows * max_rank, t.GetVMatrix(), sizeof(double) * rank * cols);
        *max_rank_out = (int) max_rank;
        return (int) rank;
    } catch (const std::exception &) {
        return -1;
    }
}

// One HCore<double>::Gemm(alpha, A, NoTrans, B, NoTrans, beta, C) (HCore.cpp:23-344).
// c_rank is read and written.  Returns 0, or -1 on an exception.
int hcref_tile_gemm(double alpha, int a_kind, int am, int an, int a_rank, int a_max_rank, double *a_data,
                    int b_kind, int bm, int bn, int b_rank, int b_max_rank, double *b_data, double beta,
                    int c_kind, int cm, int cn, int *c_rank, int c_max_rank, double *c_data, double acc,
                    int truncated, int fixed_rank, int op_type, unsigned long long *flops) {
    try {
        auto &ctx = kernels::ContextManager::GetInstance().GetContext();
        auto a = wrap_tile(a_kind, am, an, a_rank, a_max_rank, a_data, ctx);
        auto b = wrap_tile(b_kind, bm, bn, b_rank, b_max_rank, b_data, ctx);
        auto c = wrap_tile(c_kind, cm, cn, *c_rank, c_max_rank, c_data, ctx);
        auto &mh = dataunits::MemoryHandler<double>::GetInstance();
        size_t fl = 0;
        api::HCore<double>::Gemm(alpha, *a, blas::Op::NoTrans, *b, blas::Op::NoTrans, beta, *c, ctx, fl,
                                 mh.GetMemoryUnit(), make_params(acc, truncated, fixed_rank, op_type));
        if (c_kind != 0) *c_rank = (int) c->GetTileRank();
        if (flops) *flops += fl;
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// HCore<double>::Gemm with explicit operand ops and the aCholesky flag (HCore.cpp:23-344).
int hcref_tile_gemm_ops(double alpha, int a_kind, int am, int an, int a_rank, int a_max_rank, double *a_data,
                        int op_a, int b_kind, int bm, int bn, int b_rank, int b_max_rank, double *b_data, int op_b,
                        double beta, int c_kind, int cm, int cn, int *c_rank, int c_max_rank, double *c_data,
                        double acc, int truncated, int fixed_rank, int op_type, int cholesky) {
    try {
        auto &ctx = kernels::ContextManager::GetInstance().GetContext();
        auto a = wrap_tile(a_kind, am, an, a_rank, a_max_rank, a_data, ctx);
        auto b = wrap_tile(b_kind, bm, bn, b_rank, b_max_rank, b_data, ctx);
        auto c = wrap_tile(c_kind, cm, cn, *c_rank, c_max_rank, c_data, ctx);
        auto &mh = dataunits::MemoryHandler<double>::GetInstance();
        size_t fl = 0;
        api::HCore<double>::Gemm(alpha, *a, op_a ? blas::Op::Trans : blas::Op::NoTrans, *b,
                                 op_b ? blas::Op::Trans : blas::Op::NoTrans, beta, *c, ctx, fl, mh.GetMemoryUnit(),
                                 make_params(acc, truncated, fixed_rank, op_type), cholesky != 0);
        if (c_kind != 0) *c_rank = (int) c->GetTileRank();
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// HCore<double>::Potrf on a dense n x n tile (HCore.cpp:585-621).
int hcref_potrf(int uplo, int n, double *a_data) {
    try {
        auto &ctx = kernels::ContextManager::GetInstance().GetContext();
        auto a = wrap_tile(0, n, n, 0, 0, a_data, ctx);
        auto &mh = dataunits::MemoryHandler<double>::GetInstance();
        size_t fl = 0;
        api::HCore<double>::Potrf(*a, uplo ? blas::Uplo::Upper : blas::Uplo::Lower, ctx, fl, mh.GetMemoryUnit());
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// HCore<double>::Trsm with a dense n x n A and a compressed B (HCore.cpp:623-647).
int hcref_trsm(int side, int uplo, int trans, int diag, double alpha, int n, double *a_data, int bm, int bn,
               int b_rank, int b_max_rank, double *b_data) {
    try {
        auto &ctx = kernels::ContextManager::GetInstance().GetContext();
        auto a = wrap_tile(0, n, n, 0, 0, a_data, ctx);
        auto b = wrap_tile(1, bm, bn, b_rank, b_max_rank, b_data, ctx);
        auto &mh = dataunits::MemoryHandler<double>::GetInstance();
        size_t fl = 0;
        api::HCore<double>::Trsm(side ? blas::Side::Right : blas::Side::Left, uplo ? blas::Uplo::Upper : blas::Uplo::Lower,
                                 trans ? blas::Op::Trans : blas::Op::NoTrans, diag ? blas::Diag::Unit : blas::Diag::NonUnit,
                                 alpha, *a, *b, ctx, fl, mh.GetMemoryUnit());
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// HCore<double>::Syrk into a dense C (HCore.cpp:482-583); A dense (a_kind 0) or compressed (1).
int hcref_syrk(double alpha, int a_kind, int am, int an, int a_rank, int a_max_rank, double *a_data, int op_a,
               int uplo, double beta, int cm, int cn, double *c_data) {
    try {
        auto &ctx = kernels::ContextManager::GetInstance().GetContext();
        auto a = wrap_tile(a_kind, am, an, a_rank, a_max_rank, a_data, ctx);
        auto c = wrap_tile(0, cm, cn, 0, 0, c_data, ctx);
        auto &mh = dataunits::MemoryHandler<double>::GetInstance();
        size_t fl = 0;
        api::HCore<double>::Syrk(alpha, *a, op_a ? blas::Op::Trans : blas::Op::NoTrans,
                                 uplo ? blas::Uplo::Upper : blas::Uplo::Lower, beta, *c, ctx, fl, mh.GetMemoryUnit());
        return 0;
    } catch (const std::exception &) {
        return -1;
    }
}

// Tile-matrix multiply C += A*B in the style of examples/matrix_multiplication/omp_main.cpp:112-124:
// OpenMP over the listed C tiles, k ascending per C tile, one memory unit per thread.
// Tile (i, j) of an nt x nt grid is entry i + j*nt of the kind/rank/maxrank/pointer arrays.
// Only the C tiles in c_list (n_list entries of i + j*nt) are updated.  Returns seconds elapsed.
double hcref_tlr_gemm(int nt, int nb, double alpha, double beta, const int *a_kind, const int *a_rank,
                      const int *a_max_rank, double *const *a_ptr, const int *b_kind, const int *b_rank,
                      const int *b_max_rank, double *const *b_ptr, const int *c_kind, int *c_rank,
                      const int *c_max_rank, double *const *c_ptr, const int *c_list, int n_list, double acc,
                      int truncated, int fixed_rank, int op_type, int nthreads, int *errors) {
    auto &cm = kernels::ContextManager::GetInstance();
    auto &mh = dataunits::MemoryHandler<double>::GetInstance();
    const int max_units = (int) cm.GetNumOfContexts();
    if (nthreads > max_units) nthreads = max_units;
    auto params = make_params(acc, truncated, fixed_rank, op_type);
    int err = 0;
    auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(+ : err)
    for (int t = 0; t < n_list; t++) {
        int tid = omp_get_thread_num();
        auto &ctx = cm.GetContext(tid);
        int idx = c_list[t];
        int i = idx % nt, j = idx / nt;
        try {
            auto c = wrap_tile(c_kind[idx], nb, nb, c_rank[idx], c_max_rank[idx], c_ptr[idx], ctx);
            for (int k = 0; k < nt; k++) {
                int ai = i + k * nt, bi = k + j * nt;
                auto a = wrap_tile(a_kind[ai], nb, nb, a_rank[ai], a_max_rank[ai], a_ptr[ai], ctx);
                auto b = wrap_tile(b_kind[bi], nb, nb, b_rank[bi], b_max_rank[bi], b_ptr[bi], ctx);
                size_t fl = 0;
                api::HCore<double>::Gemm(alpha, *a, blas::Op::NoTrans, *b, blas::Op::NoTrans, beta, *c, ctx, fl,
                                         mh.GetMemoryUnit(tid), params);
            }
            if (c_kind[idx] != 0) c_rank[idx] = (int) c->GetTileRank();
        } catch (const std::exception &) {
            err += 1;
        }
    }
    auto t1 = std::chrono::steady_clock::now();
    if (errors) *errors = err;
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
