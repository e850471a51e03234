// hcorepp_gb300/hcore.hpp -- C++ mirror of HCore++'s TLR-GEMM API over the C ABI (hcgb.h).
//
// Same class names, namespaces, constructor arguments and call signatures as the reference for
// the tile-GEMM path, so code written against HCore++'s CUDA build recompiles against this header:
//   hcorepp::operators::CompressionParameters  include/hcorepp/operators/helpers/CompressionParameters.hpp:44-127
//   hcorepp::operators::Tile / DenseTile / CompressedTile
//                                              include/hcorepp/operators/interface/Tile.hpp:54-294,
//                                              include/hcorepp/operators/concrete/{Dense,Compressed}.hpp
//   hcorepp::kernels::RunContext               include/hcorepp/kernels/cuda/RunContext.hpp:15-53
//   hcorepp::dataunits::MemoryUnit             include/hcorepp/data-units/memory-handlers/pool/MemoryHandler.hpp:22-157
//   hcorepp::api::HCore<T>::Gemm               include/hcorepp/api/HCore.hpp:41-63
//   hcorepp::api::HCore<T>::Syrk/Potrf/Trsm    include/hcorepp/api/HCore.hpp:65-112 (src/api/HCore.cpp:482-647)
//   hcorepp::operators::TileMetadata / TilePacker  include/hcorepp/operators/interface/Tile.hpp:20-52,
//                                              include/hcorepp/operators/interface/TilePacker.hpp:17-60
// Tile buffers live on the device (as in the reference's CUDA build); constructors accept host or
// device pointers (cudaMemcpyDefault).  Errors throw std::runtime_error / std::invalid_argument as
// the reference does.  The GPU path computes in double precision: T = double.
#ifndef HCOREPP_GB300_HCORE_HPP
#define HCOREPP_GB300_HCORE_HPP

#include <cuda_runtime.h>

#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>

#include "hcgb.h"

#ifdef HCGB_HAVE_BLASPP
#include <blas.hh>
#else
namespace blas {
enum class Layout : char { ColMajor = 'C', RowMajor = 'R' };
enum class Op : char { NoTrans = 'N', Trans = 'T', ConjTrans = 'C' };
enum class Uplo : char { Upper = 'U', Lower = 'L', General = 'G' };
enum class Side : char { Left = 'L', Right = 'R' };
enum class Diag : char { NonUnit = 'N', Unit = 'U' };
}  // namespace blas
#endif

namespace hcorepp {

namespace common {
enum CompressionType { LAPACK_GESVD, LAPACK_GESDD };  // Definitions.hpp CompressionType
}

namespace detail {
inline void check(int rc, hcgb_context *ctx, const char *what) {
    if (rc == HCGB_OK || rc == HCGB_NOT_CONVERGED) return;
    std::string msg = std::string(what) + ": " + (ctx ? hcgb_last_error(ctx) : "") + " (status " +
                      std::to_string(rc) + ")";
    if (rc == HCGB_BAD_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}
inline void cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
}  // namespace detail

namespace kernels {
// One device + stream + library workspace (the CUDA RunContext's GetStream / Sync role).
class RunContext {
public:
    explicit RunContext(int device = 0, cudaStream_t stream = nullptr) {
        hcgb_context *c = nullptr;
        detail::check(hcgb_context_create(device, stream, &c), nullptr, "hcgb_context_create");
        mCtx = std::shared_ptr<hcgb_context>(c, [](hcgb_context *p) { hcgb_context_destroy(p); });
        mStream = stream;
    }
    cudaStream_t GetStream() const { return mStream; }
    void Sync() const { detail::check(hcgb_sync(mCtx.get()), mCtx.get(), "hcgb_sync"); }
    RunContext ForkChildContext() { return RunContext(*this); }
    bool SupportsOMP() const { return false; }
    hcgb_context *handle() const { return mCtx.get(); }

private:
    std::shared_ptr<hcgb_context> mCtx;
    cudaStream_t mStream;
};
}  // namespace kernels

namespace dataunits {
// A device pool with the reference's bump-allocation semantics (pool/MemoryHandler.hpp:22-157,
// src/data-units/memory-handlers/pool/MemoryHandler.cpp:20-50): Initialize allocates and zeroes it,
// RequestAllocation hands out consecutive slices and throws when the pool is exhausted or not
// initialised, Reset rewinds (zeroing the pool on the context stream), Free releases it.  HCore<T>'s
// operations here take their scratch from the library's per-context workspace instead, so a unit
// serves callers that carve their own temporaries (the reference's examples and tests do).
template <typename T>
class MemoryUnit {
public:
    explicit MemoryUnit(const kernels::RunContext &ctx, size_t aAllocationSize = 0) : mCtx(&ctx) {
        if (aAllocationSize > 0) Initialize(aAllocationSize);
    }
    MemoryUnit(const MemoryUnit &) = delete;
    MemoryUnit &operator=(const MemoryUnit &) = delete;
    ~MemoryUnit() { Free(); }

    T *RequestAllocation(size_t aSize) {
        if (mAvailable < aSize || mpData == nullptr)
            throw std::runtime_error("Requested Allocation Greater than MemoryUnit Size or the pool isn't initialized");
        T *ret = mpData + mNext;
        mNext += aSize;
        mAvailable -= aSize;
        return ret;
    }
    T *GetData() const { return mpData; }
    size_t GetPoolSize() const { return mSize; }
    size_t GetPoolAvailableSize() const { return mAvailable; }
    bool IsInitialized() const { return mpData != nullptr; }
    void Initialize(size_t aSize) {
        if (IsInitialized()) throw std::runtime_error("MemoryUnit Is Already Allocated");
        if (aSize == 0) return;
        detail::cuda(cudaMalloc(reinterpret_cast<void **>(&mpData), sizeof(T) * aSize), "MemoryUnit::Initialize");
        mSize = mAvailable = aSize;
        mNext = 0;
        BufferMemSet(0, aSize);
    }
    void BufferMemSet(char aValue, size_t aSize, size_t aOffset = 0) {
        if (mpData)
            detail::cuda(cudaMemsetAsync(mpData + aOffset, aValue, sizeof(T) * aSize, mCtx->GetStream()),
                         "MemoryUnit::BufferMemSet");
    }
    void Free() {
        if (!mpData) return;
        cudaStreamSynchronize(mCtx->GetStream());
        cudaFree(mpData);
        mpData = nullptr;
        mSize = mAvailable = mNext = 0;
    }
    void FreeAllocations() { Free(); }
    void Reset() {
        mAvailable = mSize;
        mNext = 0;
        if (mpData) BufferMemSet(0, mSize);
    }

private:
    const kernels::RunContext *mCtx = nullptr;
    T *mpData = nullptr;
    size_t mSize = 0, mAvailable = 0, mNext = 0;
};
}  // namespace dataunits

namespace operators {

class CompressionParameters {
public:
    CompressionParameters(double aAccuracy = 1e-4, bool aUseTrmm = false, bool aUseUngqr = true,
                          bool aTruncatedSvd = false, size_t aFixedRank = 0,
                          common::CompressionType aOpType = common::LAPACK_GESDD)
        : mUseTrmm(aUseTrmm), mUseUngqr(aUseUngqr), mTruncatedSvd(aTruncatedSvd), mFixedRank(aFixedRank),
          mOpType(aOpType), mAccuracy(aAccuracy) {}
    bool GetTrmm() const { return mUseTrmm; }
    bool GetUngqr() const { return mUseUngqr; }
    bool GetTruncatedSvd() const { return mTruncatedSvd; }
    size_t GetFixedRank() const { return mFixedRank; }
    common::CompressionType GetOperationType() const { return mOpType; }
    double GetAccuracy() const { return mAccuracy; }
    // GB300 addition: arithmetic of the recompression core (HCGB_PLAIN_FP64 or HCGB_MIXED).
    void SetMode(int aMode) { mMode = aMode; }
    hcgb_params c_params() const {
        return hcgb_params{mAccuracy, mTruncatedSvd ? 1 : 0, (int) mFixedRank, mUseTrmm ? 1 : 0,
                           mUseUngqr ? 1 : 0, mOpType == common::LAPACK_GESVD ? HCGB_GESVD : HCGB_GESDD, mMode};
    }

private:
    bool mUseTrmm, mUseUngqr, mTruncatedSvd;
    size_t mFixedRank;
    common::CompressionType mOpType;
    double mAccuracy;
    int mMode = HCGB_PLAIN_FP64;
};

// Tile metadata for task runtimes moving tiles between workers (Tile.hpp:20-52): everything but
// the data buffer, which stays where it is (device memory) and travels as one pointer.
enum TileType { DENSE, COMPRESSED };

struct TileMetadata {
    size_t mNumOfRows;
    size_t mNumOfCols;
    size_t mMatrixRank;
    size_t mMaxRank;
    size_t mLeadingDimension;
    blas::Layout mLayout;
    TileType mType;
    TileMetadata(size_t aRows, size_t aCols, size_t aMatrixRank, size_t aMaxRank, size_t aLeadingDim,
                 blas::Layout aLayout, TileType aType)
        : mNumOfRows(aRows), mNumOfCols(aCols), mMatrixRank(aMatrixRank), mMaxRank(aMaxRank),
          mLeadingDimension(aLeadingDim), mLayout(aLayout), mType(aType) {}
};

template <typename T>
class Tile {
public:
    static_assert(sizeof(T) == 8, "the GB300 TLR path computes in double precision");
    virtual ~Tile() = default;
    // (metadata, data buffer) of this tile; the metadata is heap-allocated and owned by the caller,
    // the buffer stays owned by the tile (Dense.cpp:127-134, Compressed.cpp:769-778).
    virtual std::pair<TileMetadata *, T *> UnPackTile(const kernels::RunContext &aContext) = 0;
    // Re-point this tile at a buffer described by aMetadata, without copying; the tile does not own
    // the buffer afterwards (Dense.cpp:136-142, Compressed.cpp:780-788).
    virtual void PackTile(TileMetadata aMetadata, T *aDataArray, const kernels::RunContext &aContext) = 0;
    size_t GetNumOfRows() const { return mRows; }
    size_t GetNumOfCols() const { return mCols; }
    blas::Layout GetLayout() const { return blas::Layout::ColMajor; }
    virtual int GetNumOfSubMatrices() const = 0;
    virtual size_t GetTileRank() const = 0;
    virtual hcgb_tile c_tile() const = 0;
    bool isDense() const { return GetNumOfSubMatrices() == 1; }
    bool isCompressed() const { return GetNumOfSubMatrices() == 2; }

protected:
    size_t mRows = 0, mCols = 0;
};

template <typename T>
class DenseTile : public Tile<T> {
public:
    // DenseTile(rows, cols, data, ld, layout, ctx, owning) (Dense.hpp:90-91).  With owning = false
    // the tile wraps the caller's DEVICE buffer; otherwise the data (host or device) is copied.
    DenseTile(size_t aRows, size_t aCols, T *aData, size_t aLd, blas::Layout aLayout,
              const kernels::RunContext &aContext, bool aOwning = true) {
        if (aLayout != blas::Layout::ColMajor) throw std::invalid_argument("DenseTile: column-major only");
        this->mRows = aRows;
        this->mCols = aCols;
        if (!aOwning) {
            mData = aData;
            return;
        }
        detail::cuda(cudaMalloc(&mData, sizeof(T) * aRows * aCols), "cudaMalloc");
        mOwn = true;
        if (aData)
            detail::cuda(cudaMemcpy2D(mData, sizeof(T) * aRows, aData, sizeof(T) * aLd, sizeof(T) * aRows, aCols,
                                      cudaMemcpyDefault),
                         "cudaMemcpy2D");
        else
            detail::cuda(cudaMemset(mData, 0, sizeof(T) * aRows * aCols), "cudaMemset");
    }
    DenseTile(size_t aRows, size_t aCols, T *aData, size_t aLd, const kernels::RunContext &aContext)
        : DenseTile(aRows, aCols, aData, aLd, blas::Layout::ColMajor, aContext) {}
    DenseTile() = default;
    std::pair<TileMetadata *, T *> UnPackTile(const kernels::RunContext &) override {
        return {new TileMetadata(this->mRows, this->mCols, 0, 0, this->mRows, blas::Layout::ColMajor, DENSE), mData};
    }
    void PackTile(TileMetadata aMetadata, T *aDataArray, const kernels::RunContext &) override {
        if (aMetadata.mType != DENSE || aMetadata.mLayout != blas::Layout::ColMajor ||
            aMetadata.mLeadingDimension != aMetadata.mNumOfRows)
            throw std::invalid_argument("DenseTile::PackTile: column-major dense metadata with ld = rows expected");
        if (mOwn) cudaFree(mData);
        mOwn = false;
        mData = aDataArray;
        this->mRows = aMetadata.mNumOfRows;
        this->mCols = aMetadata.mNumOfCols;
    }
    ~DenseTile() override {
        if (mOwn) cudaFree(mData);
    }
    DenseTile(const DenseTile &) = delete;
    DenseTile &operator=(const DenseTile &) = delete;
    int GetNumOfSubMatrices() const override { return 1; }
    size_t GetTileRank() const override { return 0; }
    T *GetTileSubMatrix(size_t aIndex) const {
        if (aIndex != 0) throw std::invalid_argument("GetTileSubMatrix ::Index out of range");
        return mData;
    }
    size_t GetLeadingDim() const { return this->mRows; }
    hcgb_tile c_tile() const override {
        return hcgb_tile{mData, nullptr, (int) this->mRows, (int) this->mCols, 0, HCGB_DENSE};
    }

private:
    T *mData = nullptr;
    bool mOwn = false;
};

template <typename T>
class CompressedTile : public Tile<T> {
public:
    // (rows, cols, data, ld, rank, layout, ctx) (Compressed.cpp:50-73): data = packed [U | V],
    // max rank = rank (the rank can never grow).
    CompressedTile(size_t aRows, size_t aCols, T *aData, size_t aLd, size_t aRank, blas::Layout aLayout,
                   const kernels::RunContext &aContext) {
        init(aRows, aCols, aRank, aRank);
        if (aData) {
            detail::cuda(cudaMemcpy(mData, aData, sizeof(T) * aRows * aRank, cudaMemcpyDefault), "cudaMemcpy");
            detail::cuda(cudaMemcpy(GetVMatrix(), aData + aRows * aRank, sizeof(T) * aRank * aCols,
                                    cudaMemcpyDefault),
                         "cudaMemcpy");
        }
        set_rank(aRank);
    }
    CompressedTile(size_t aRows, size_t aCols, T *aData, size_t aLd, size_t aRank,
                   const kernels::RunContext &aContext)
        : CompressedTile(aRows, aCols, aData, aLd, aRank, blas::Layout::ColMajor, aContext) {}
    // (rows, cols, dense data, ld, params, layout, ctx) (Compressed.cpp:75-146): truncated SVD on
    // the GPU, max rank = max(min(rows, cols) / 3, 1).
    CompressedTile(size_t aRows, size_t aCols, T *aData, size_t aLd, const CompressionParameters &aParameters,
                   blas::Layout aLayout, const kernels::RunContext &aContext) {
        const size_t maxr = std::max<size_t>(std::min(aRows, aCols) / 3, 1);
        init(aRows, aCols, maxr, 0);
        if (aData) {
            T *dd = nullptr;
            detail::cuda(cudaMalloc(&dd, sizeof(T) * aRows * aCols), "cudaMalloc");
            detail::cuda(cudaMemcpy2D(dd, sizeof(T) * aRows, aData, sizeof(T) * aLd, sizeof(T) * aRows, aCols,
                                      cudaMemcpyDefault),
                         "cudaMemcpy2D");
            hcgb_tile t = c_tile();
            hcgb_params p = aParameters.c_params();
            int r = 0;
            int rc = hcgb_compress_tile(aContext.handle(), dd, (int) aRows, (int) aCols, &t, &p, &r);
            cudaFree(dd);
            detail::check(rc, aContext.handle(), "hcgb_compress_tile");
        }
    }
    CompressedTile() = default;
    ~CompressedTile() override {
        if (mOwnData) cudaFree(mData);
        cudaFree(mRank);
    }
    std::pair<TileMetadata *, T *> UnPackTile(const kernels::RunContext &) override {
        return {new TileMetadata(this->mRows, this->mCols, GetTileRank(), mMaxRank, this->mRows,
                                 blas::Layout::ColMajor, COMPRESSED),
                mData};
    }
    void PackTile(TileMetadata aMetadata, T *aDataArray, const kernels::RunContext &) override {
        if (aMetadata.mType != COMPRESSED || aMetadata.mLayout != blas::Layout::ColMajor ||
            aMetadata.mMatrixRank > aMetadata.mMaxRank)
            throw std::invalid_argument("CompressedTile::PackTile: column-major compressed metadata expected");
        if (mOwnData) cudaFree(mData);
        mOwnData = false;
        mData = aDataArray;
        this->mRows = aMetadata.mNumOfRows;
        this->mCols = aMetadata.mNumOfCols;
        mMaxRank = aMetadata.mMaxRank;
        if (!mRank) detail::cuda(cudaMalloc(&mRank, sizeof(int)), "cudaMalloc");
        set_rank(aMetadata.mMatrixRank);
    }
    CompressedTile(const CompressedTile &) = delete;
    CompressedTile &operator=(const CompressedTile &) = delete;
    int GetNumOfSubMatrices() const override { return 2; }
    size_t GetTileRank() const override {
        int r = 0;
        detail::cuda(cudaMemcpy(&r, mRank, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        return (size_t) r;
    }
    T *GetUMatrix() const { return mData; }
    T *GetVMatrix() const { return mData + this->mRows * mMaxRank; }
    size_t GetULeadingDim() const { return this->mRows; }
    size_t GetVLeadingDim() const { return GetTileRank(); }
    size_t GetMaxRank() const { return mMaxRank; }
    T *GetTileSubMatrix(size_t aIndex) const {
        if (aIndex > 1) throw std::invalid_argument("CompressedTile::GetTileSubMatrix:: Index out of range");
        return aIndex == 0 ? GetUMatrix() : GetVMatrix();
    }
    int *GetDeviceRank() const { return mRank; }
    hcgb_tile c_tile() const override {
        return hcgb_tile{mData, mRank, (int) this->mRows, (int) this->mCols, (int) mMaxRank, HCGB_COMPRESSED};
    }
    // The Cholesky-flow reading of the same buffer: V region = W = V^T (cols x rank, ld cols).
    hcgb_tile c_tile_vt() const {
        hcgb_tile t = c_tile();
        t.kind = HCGB_COMPRESSED_VT;
        return t;
    }
    // Room for the full-rank form a DDC update produces (HCore.cpp:294-298 re-sizes the tile the
    // same way): grow the buffer to rank min(rows, cols), keeping U and V in place.
    void EnsureFullRankCapacity() {
        const size_t r = std::min(this->mRows, this->mCols);
        if (r <= mMaxRank) return;
        const size_t rank = GetTileRank();
        T *nd = nullptr;
        const size_t cap = this->mRows * r + r * this->mCols;
        detail::cuda(cudaMalloc(&nd, sizeof(T) * cap), "cudaMalloc");
        detail::cuda(cudaMemset(nd, 0, sizeof(T) * cap), "cudaMemset");
        detail::cuda(cudaMemcpy(nd, mData, sizeof(T) * this->mRows * rank, cudaMemcpyDeviceToDevice), "cudaMemcpy");
        detail::cuda(cudaMemcpy(nd + this->mRows * r, GetVMatrix(), sizeof(T) * rank * this->mCols,
                                cudaMemcpyDeviceToDevice),
                     "cudaMemcpy");
        if (mOwnData) cudaFree(mData);
        mData = nd;
        mOwnData = true;
        mMaxRank = r;
    }

private:
    void init(size_t rows, size_t cols, size_t maxr, size_t rank) {
        this->mRows = rows;
        this->mCols = cols;
        mMaxRank = maxr;
        const size_t cap = rows * maxr + maxr * cols;
        detail::cuda(cudaMalloc(&mData, sizeof(T) * cap), "cudaMalloc");
        detail::cuda(cudaMemset(mData, 0, sizeof(T) * cap), "cudaMemset");
        detail::cuda(cudaMalloc(&mRank, sizeof(int)), "cudaMalloc");
        set_rank(rank);
    }
    void set_rank(size_t r) {
        int v = (int) r;
        detail::cuda(cudaMemcpy(mRank, &v, sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    T *mData = nullptr;
    int *mRank = nullptr;
    size_t mMaxRank = 0;
    bool mOwnData = true;
};

// TilePacker (TilePacker.hpp:17-60, src/operators/TilePacker.cpp:5-26).
template <typename T>
class TilePacker {
public:
    virtual ~TilePacker() = default;
    static std::pair<TileMetadata *, T *> UnPackTile(Tile<T> &aTile, const kernels::RunContext &aContext) {
        return aTile.UnPackTile(aContext);
    }
    // A new heap tile (owned by the caller) over the given buffer.
    static Tile<T> *PackTile(TileMetadata aMetadata, T *aDataArray, const kernels::RunContext &aContext) {
        Tile<T> *tile;
        if (aMetadata.mType == DENSE) tile = new DenseTile<T>();
        else tile = new CompressedTile<T>();
        tile->PackTile(aMetadata, aDataArray, aContext);
        return tile;
    }
};

}  // namespace operators

namespace api {

template <typename T>
class HCore {
public:
    // C = alpha op(A) op(B) + beta C (HCore.cpp:23-344); flops += the reference's count.
    static void Gemm(T aAlpha, const operators::Tile<T> &aA, const blas::Op &aAOp, const operators::Tile<T> &aB,
                     const blas::Op &aBOp, T aBeta, operators::Tile<T> &aC, const kernels::RunContext &aContext,
                     size_t &aFlops, dataunits::MemoryUnit<T> &aMemoryUnit,
                     const operators::CompressionParameters &aParameters = {1e-9}, bool aCholesky = false) {
        hcgb_tile a = aA.c_tile(), b = aB.c_tile(), c = aC.c_tile();
        if (aCholesky) {
            // The aCholesky branch (HCore.cpp:160-174, Compressed.cpp:273-276, :529-595, :669-673):
            // compressed A, B, C whose V regions hold W = V^T, op(A) = NoTrans, op(B) = Trans.  The
            // reference's branch gives no meaningful result for other combinations; they are rejected.
            if (!aA.isCompressed() || !aB.isCompressed() || !aC.isCompressed() || aAOp != blas::Op::NoTrans ||
                aBOp == blas::Op::NoTrans)
                throw std::invalid_argument("HCore::Gemm(aCholesky): compressed A, B, C with NoTrans, Trans only");
            a = static_cast<const operators::CompressedTile<T> &>(aA).c_tile_vt();
            b = static_cast<const operators::CompressedTile<T> &>(aB).c_tile_vt();
            c = static_cast<operators::CompressedTile<T> &>(aC).c_tile_vt();
        } else if (aA.isDense() && aB.isDense() && aC.isCompressed()) {
            // The DDC combination re-sets C at full rank: make room first.
            static_cast<operators::CompressedTile<T> &>(aC).EnsureFullRankCapacity();
            c = aC.c_tile();
        }
        hcgb_params p = aParameters.c_params();
        int r = 0;
        unsigned long long fl = 0;
        const int oa = aAOp == blas::Op::NoTrans ? HCGB_NOTRANS : HCGB_TRANS;
        const int ob = aBOp == blas::Op::NoTrans ? HCGB_NOTRANS : HCGB_TRANS;
        detail::check(hcgb_tile_gemm(aContext.handle(), aAlpha, &a, oa, &b, ob, aBeta, &c, &p, &r, &fl),
                      aContext.handle(), "HCore::Gemm");
        aFlops += (size_t) fl;
    }

    // Syrk (HCore.cpp:482-583) into a dense C.  Dense A: dsyrk(uplo, op, n, k = C.cols) on the uplo
    // triangle.  Compressed A read as U W^T: C <- beta C - A A^T (the reference uses -1, not alpha),
    // then the opposite strict triangle is set to zero (FillMatrixTriangle).
    static void Syrk(T aAlpha, const operators::Tile<T> &aA, const blas::Op &aAOp, blas::Uplo aUplo, T aBeta,
                     operators::Tile<T> &aC, const kernels::RunContext &aContext, size_t &aFlops,
                     dataunits::MemoryUnit<T> &aMemoryUnit) {
        if (!aC.isDense()) throw std::invalid_argument("HCore::Syrk: C must be dense");
        hcgb_tile c = aC.c_tile();
        const int lo = aUplo == blas::Uplo::Upper ? HCGB_UPPER : HCGB_LOWER;
        if (aA.isDense()) {
            hcgb_tile a = aA.c_tile();
            const int op = aAOp == blas::Op::NoTrans ? HCGB_NOTRANS : HCGB_TRANS;
            detail::check(hcgb_syrk(aContext.handle(), lo, op, c.rows, c.cols, aAlpha, a.data, a.rows, aBeta, c.data,
                                    c.rows),
                          aContext.handle(), "HCore::Syrk");
            return;
        }
        hcgb_tile a = static_cast<const operators::CompressedTile<T> &>(aA).c_tile_vt();
        hcgb_params p = operators::CompressionParameters(1e-9).c_params();
        unsigned long long fl = 0;
        detail::check(hcgb_tile_gemm(aContext.handle(), -1.0, &a, HCGB_NOTRANS, &a, HCGB_TRANS, aBeta, &c, &p,
                                     nullptr, &fl),
                      aContext.handle(), "HCore::Syrk");
        detail::check(hcgb_fill_triangle(aContext.handle(), lo == HCGB_LOWER ? HCGB_UPPER : HCGB_LOWER, c.rows,
                                         c.data, c.rows, 0.0),
                      aContext.handle(), "HCore::Syrk");
        aFlops += (size_t) fl;
    }

    // Potrf (HCore.cpp:585-621): dense tiles only; dpotrf semantics on the uplo triangle.
    static void Potrf(operators::Tile<T> &aA, blas::Uplo aUplo, const kernels::RunContext &aContext,
                      size_t &aFlops, dataunits::MemoryUnit<T> &aMemoryUnit) {
        if (aA.GetNumOfSubMatrices() != 1) throw std::runtime_error(" Potrf works only with dense tiles");
        hcgb_tile a = aA.c_tile();
        int info = 0;
        detail::check(hcgb_potrf(aContext.handle(), aUplo == blas::Uplo::Upper ? HCGB_UPPER : HCGB_LOWER, a.rows,
                                 a.data, a.rows, &info),
                      aContext.handle(), "HCore::Potrf");
    }

    // Trsm (HCore.cpp:623-647): B compressed; the solve runs on its V region read as rows x rank
    // (ld rows), i.e. on W of the Cholesky-flow layout.
    static void Trsm(blas::Side aSide, blas::Uplo aUplo, blas::Op aTrans, blas::Diag aDiag, T aAlpha,
                     operators::Tile<T> &aA, operators::Tile<T> &aB, const kernels::RunContext &aContext,
                     size_t &aFlops, dataunits::MemoryUnit<T> &aMemoryHandler) {
        if (aB.GetNumOfSubMatrices() != 2) throw std::runtime_error(" TRSM: Tile B must be compressed ");
        auto &b = static_cast<operators::CompressedTile<T> &>(aB);
        hcgb_tile a = aA.c_tile();
        detail::check(hcgb_trsm(aContext.handle(), aSide == blas::Side::Right ? HCGB_RIGHT : HCGB_LEFT,
                                aUplo == blas::Uplo::Upper ? HCGB_UPPER : HCGB_LOWER,
                                aTrans == blas::Op::NoTrans ? HCGB_NOTRANS : HCGB_TRANS,
                                aDiag == blas::Diag::Unit ? HCGB_UNIT : HCGB_NONUNIT, (int) b.GetNumOfRows(),
                                (int) b.GetTileRank(), aAlpha, a.data, a.rows, b.GetVMatrix(), (int) b.GetNumOfRows()),
                      aContext.handle(), "HCore::Trsm");
    }

    // Scratch the library needs for one update of these tiles (HCore.cpp:417-480), in elements of T.
    static size_t CalculateMemoryPoolSize(const operators::Tile<T> &aA, const operators::Tile<T> &aB,
                                          const operators::Tile<T> &aC, operators::CompressionParameters,
                                          const kernels::RunContext &) {
        hcgb_tile a = aA.c_tile(), b = aB.c_tile(), c = aC.c_tile();
        const int rab = std::max(a.kind != HCGB_DENSE ? a.max_rank : 0, b.kind != HCGB_DENSE ? b.max_rank : 0);
        return hcgb_workspace_bytes(1, (int) std::max(c.rows, a.cols), c.cols,
                                    c.kind != HCGB_DENSE ? c.max_rank : 0, rab) / sizeof(T);
    }
};

}  // namespace api
}  // namespace hcorepp

#endif  // HCOREPP_GB300_HCORE_HPP
