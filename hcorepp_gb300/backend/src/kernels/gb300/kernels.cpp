/*
 * HCoreKernels<T> of the GB300 backend: the static kernels HCore++'s operators call
 * (include/hcorepp/kernels/kernels.hpp:24-137), on libhcgb's device kernels (include/hcgb.h).
 * Replaces src/kernels/cuda/kernels.cpp (cuBLAS / cuSOLVER calls) and CudaKernels.cu for a
 * USE_GB300 build; the reference's own operators (CompressedTile<T>::Gemm's step-by-step
 * recompression, Compressed.cpp:208-694) then run unchanged on GB300.  For whole tile matrices
 * and batches, hcgb_tlr_gemm / hcgb_gemm_batch are the fast path.
 *
 * T = double only: libhcgb computes in FP64.  Every HCoreKernels<float> entry throws
 * std::runtime_error (the reference instantiates float too, include/hcorepp/common/Definitions.hpp:10-11).
 * Column-major layouts (the only ones the reference's TLR path uses); a row-major call throws,
 * except where the operation is layout-symmetric.  libhcgb errors throw std::runtime_error with
 * the context's message, as the reference's LAPACK++ / error-check paths throw or abort.
 */
#include <hcorepp/kernels/kernels.hpp>

#include <stdexcept>
#include <string>
#include <vector>

namespace hcorepp {
    namespace kernels {
        namespace {
            void Check(int aStatus, const RunContext &aContext, const char *apWhat) {
                if (aStatus != HCGB_OK) {
                    throw std::runtime_error(std::string("GB300 ") + apWhat + ": " +
                                             hcgb_last_error(aContext.GetHcgbContext()));
                }
            }

            void ColMajorOnly(blas::Layout aLayout, const char *apWhat) {
                if (aLayout != blas::Layout::ColMajor) {
                    throw std::runtime_error(std::string("GB300 ") + apWhat + ": column-major layout only");
                }
            }

            int Trans(blas::Op aOp) {
                return aOp == blas::Op::NoTrans ? HCGB_NOTRANS : HCGB_TRANS;
            }

            int Uplo(blas::Uplo aUplo) {
                return aUplo == blas::Uplo::Upper ? HCGB_UPPER : HCGB_LOWER;
            }

            int Part(common::MatrixType aType) {
                switch (aType) {
                    case common::MatrixType::General:
                        return HCGB_PART_GENERAL;
                    case common::MatrixType::Upper:
                        return HCGB_PART_UPPER;
                    case common::MatrixType::Lower:
                        return HCGB_PART_LOWER;
                    default:
                        throw std::runtime_error("GB300 lacpy/laset: general, upper or lower matrices only");
                }
            }

            int SvdJob(common::Job aJob) {
                if (aJob == common::Job::NoVec) return HCGB_SVD_NONE;
                if (aJob == common::Job::SomeVec) return HCGB_SVD_SOME;
                if (aJob == common::Job::AllVec) return HCGB_SVD_ALL;
                throw std::runtime_error("GB300 SVD: NoVec, SomeVec or AllVec only");
            }

            int I(size_t aValue) {
                return static_cast<int>(aValue);
            }

            [[noreturn]] void FloatUnsupported(const char *apWhat) {
                throw std::runtime_error(std::string("GB300 backend: ") + apWhat +
                                         " is FP64 only (HCoreKernels<float> unsupported)");
            }
        }

        // ------------------------------------------------------------------ double
        template<>
        void HCoreKernels<double>::Gemm(blas::Layout aLayout, blas::Op aTransA, blas::Op aTransB, size_t aM,
                                        size_t aN, size_t aK, double &aAlpha, double const *apA, size_t aLdA,
                                        double const *apB, size_t aLdB, double &aBeta, double *apC, size_t aLdC,
                                        const RunContext &aContext) {
            int rc;
            if (aLayout == blas::Layout::ColMajor) {
                rc = hcgb_dgemm(aContext.GetHcgbContext(), Trans(aTransA), Trans(aTransB), I(aM), I(aN), I(aK),
                                aAlpha, apA, I(aLdA), apB, I(aLdB), aBeta, apC, I(aLdC));
            } else {  // row-major C = op(A) op(B)  <=>  column-major C^T = op(B)^T op(A)^T
                rc = hcgb_dgemm(aContext.GetHcgbContext(), Trans(aTransB), Trans(aTransA), I(aN), I(aM), I(aK),
                                aAlpha, apB, I(aLdB), apA, I(aLdA), aBeta, apC, I(aLdC));
            }
            Check(rc, aContext, "Gemm");
        }

        template<>
        void HCoreKernels<double>::MultiplyByAlpha(double *apArray, size_t aRows, size_t aCols, size_t aM,
                                                   size_t aRank, double &aAlpha, const RunContext &aContext) {
            const int count = I(aRows * aCols);
            double *p = apArray + aM * aRank;
            Check(hcgb_dcopy2d(aContext.GetHcgbContext(), 0, count, 1, aAlpha, p, count, p, count), aContext,
                  "MultiplyByAlpha");
        }

        template<>
        void HCoreKernels<double>::ProcessVpointer(size_t aN, size_t aCRank, bool aGetUngqr, size_t Vm,
                                                   double &aBeta, double *apCV, size_t aLdcV, double *V,
                                                   size_t aArank, const double *apBdata,
                                                   const RunContext &aContext, bool aCholesky) {
            hcgb_context *c = aContext.GetHcgbContext();
            double *Vptr = &V[aN * aCRank];
            if (aCholesky) {
                Check(hcgb_dcopy2d(c, 0, I(aCRank), I(aN), aBeta, apCV, I(aLdcV), V, I(aLdcV)), aContext,
                      "ProcessVpointer");
                Check(hcgb_dcopy2d(c, 0, I(aArank), I(aN), 1.0, apBdata, I(aArank), Vptr, I(aArank)), aContext,
                      "ProcessVpointer");
            } else {
                // V[:, :CRank] = beta Cv^T (Vm rows), then the next columns = B^T
                Check(hcgb_dcopy2d(c, 1, I(aN), I(aCRank), aBeta, apCV, I(aLdcV), V, I(Vm)), aContext,
                      "ProcessVpointer");
                Check(hcgb_dcopy2d(c, 1, I(aN), I(aArank), 1.0, apBdata, I(aArank), Vptr, I(Vm)), aContext,
                      "ProcessVpointer");
            }
        }

        template<>
        void HCoreKernels<double>::CalculateNewRank(size_t &aNewRank, bool aTruncatedSvd, double *apSigma,
                                                    size_t sizeS, double accuracy, const RunContext &aContext) {
            // The singular values are device memory (the SVD's output): one read, then the reference's
            // rule (src/kernels/omp/kernels.cpp:82-104).
            std::vector<double> s(sizeS);
            if (sizeS) {
                if (cudaMemcpyAsync(s.data(), apSigma, sizeof(double) * sizeS, cudaMemcpyDefault,
                                    aContext.GetStream()) != cudaSuccess ||
                    cudaStreamSynchronize(aContext.GetStream()) != cudaSuccess) {
                    throw std::runtime_error("GB300 CalculateNewRank: reading the singular values failed");
                }
            }
            aNewRank = sizeS;
            for (size_t i = 1; i < sizeS; i++) {
                if (s[i] < (aTruncatedSvd ? accuracy * s[0] : accuracy)) {
                    aNewRank = i;
                    break;
                }
            }
        }

        template<>
        void HCoreKernels<double>::CalculateUVptr(size_t aRank, size_t aVm, double *UVptr, const double *Vnew,
                                                  const RunContext &aContext) {
            Check(hcgb_dcopy2d(aContext.GetHcgbContext(), 1, I(aRank), I(aVm), 1.0, Vnew, I(aVm), UVptr, I(aRank)),
                  aContext, "CalculateUVptr");
        }

        template<>
        void HCoreKernels<double>::CalculateVTnew(size_t aRkNew, bool aUngqr, size_t aMinVmVn, double *apSigma,
                                                  double *apVTnew, size_t aSizeS, size_t aVm,
                                                  const RunContext &aContext) {
            Check(hcgb_dscale_rows(aContext.GetHcgbContext(), I(aRkNew), I(aUngqr ? aMinVmVn : aVm), apSigma,
                                   apVTnew, I(aSizeS)), aContext, "CalculateVTnew");
        }

        template<>
        void HCoreKernels<double>::CalculateUVptrConj(size_t aRank, size_t aVm, double *UVptr,
                                                      const RunContext &aContext) {
            // real arithmetic: conjugation is the identity
        }

        template<>
        void HCoreKernels<double>::FillIdentityMatrix(size_t aNumOfElements, double *apMatrix,
                                                      const RunContext &aContext) {
            const int n = I(aNumOfElements);
            Check(hcgb_dlaset(aContext.GetHcgbContext(), HCGB_PART_DIAGONAL, n, n, 0.0, 1.0, apMatrix, n), aContext,
                  "FillIdentityMatrix");
        }

        template<>
        void HCoreKernels<double>::LaCpy(common::MatrixType aType, size_t aM, size_t aRank, double *apCU, size_t aLD,
                                         double *apU, size_t aUm, const RunContext &aContext) {
            Check(hcgb_dlacpy(aContext.GetHcgbContext(), Part(aType), I(aM), I(aRank), apCU, I(aLD), apU, I(aUm)),
                  aContext, "LaCpy");
        }

        template<>
        void HCoreKernels<double>::Geqrf(size_t aM, size_t aN, double *apA, size_t aLdA, double *apTau,
                                         double *aWorkspace, size_t aWorkspace_size, size_t aHostSize,
                                         const RunContext &aContext) {
            Check(hcgb_dgeqrf(aContext.GetHcgbContext(), I(aM), I(aN), apA, I(aLdA), apTau), aContext, "Geqrf");
        }

        template<>
        void HCoreKernels<double>::Laset(common::MatrixType aMatrixType, size_t aM, size_t aN, double aOffdiag,
                                         double aDiag, double *apA, size_t aLdA, const RunContext &aContext) {
            Check(hcgb_dlaset(aContext.GetHcgbContext(), Part(aMatrixType), I(aM), I(aN), aOffdiag, aDiag, apA,
                              I(aLdA)), aContext, "Laset");
        }

        template<>
        void HCoreKernels<double>::Trmm(blas::Layout aLayout, blas::Side aSide, blas::Uplo aUplo, blas::Op aTrans,
                                        blas::Diag aDiag, size_t aM, size_t aN, double aAlpha, double const *apA,
                                        size_t aLdA, double *apB, size_t aLdB, const RunContext &aContext) {
            ColMajorOnly(aLayout, "Trmm");
            Check(hcgb_dtrmm(aContext.GetHcgbContext(), aSide == blas::Side::Left ? HCGB_LEFT : HCGB_RIGHT,
                             Uplo(aUplo), Trans(aTrans), aDiag == blas::Diag::Unit ? HCGB_UNIT : HCGB_NONUNIT,
                             I(aM), I(aN), aAlpha, apA, I(aLdA), apB, I(aLdB)), aContext, "Trmm");
        }

        template<>
        void HCoreKernels<double>::SVD(common::Job aJobu, common::Job aJobvt, size_t aM, size_t aN, double *apA,
                                       size_t aLdA, double *apS, double *apU, size_t aLdU, double *apVT,
                                       size_t aLdVt, common::CompressionType aSVDType, double *aWorkspace,
                                       size_t aWorkspace_size, size_t aHostSize, const RunContext &aContext) {
            // gesdd takes one job for both factors (the reference passes aJobu, kernels/omp/kernels.cpp:188-190)
            const int ju = SvdJob(aJobu);
            const int jv = aSVDType == common::CompressionType::LAPACK_GESDD ? ju : SvdJob(aJobvt);
            int info = 0;
            Check(hcgb_dgesvd(aContext.GetHcgbContext(), ju, jv, I(aM), I(aN), apA, I(aLdA), apS, apU, I(aLdU), apVT,
                              I(aLdVt), &info), aContext, "SVD");
        }

        template<>
        void HCoreKernels<double>::Unmqr(common::SideMode aSide, common::BlasOperation aTrans, size_t aM, size_t aN,
                                         size_t aK, double const *apA, size_t aLdA, double const *apTau, double *apC,
                                         size_t aLdC, double *aWorkspace, size_t aWorkspace_size,
                                         const RunContext &aContext) {
            Check(hcgb_dormqr(aContext.GetHcgbContext(), aSide == common::SIDE_LEFT ? HCGB_LEFT : HCGB_RIGHT,
                              aTrans == common::OP_NoTRANS ? HCGB_NOTRANS : HCGB_TRANS, I(aM), I(aN), I(aK), apA,
                              I(aLdA), apTau, apC, I(aLdC)), aContext, "Unmqr");
        }

        template<>
        void HCoreKernels<double>::ungqr(size_t aM, size_t aN, size_t aK, double *apA, size_t aLdA, double *apTau,
                                         double *aWorkspace, size_t aWorkspace_size, const RunContext &aContext) {
            Check(hcgb_dorgqr(aContext.GetHcgbContext(), I(aM), I(aN), I(aK), apA, I(aLdA), apTau), aContext,
                  "ungqr");
        }

        template<>
        size_t HCoreKernels<double>::CalculateGemmWorkspaceSize(size_t aUm, size_t aUn, size_t aVm, size_t aVn,
                                                                size_t aSizeS,
                                                                const operators::CompressionParameters &aHelpers,
                                                                size_t &aHostSize, const RunContext &aContext) {
            aHostSize = 0;  // the kernels keep their scratch in the libhcgb context
            return 0;
        }

        template<>
        int HCoreKernels<double>::potrf(blas::Uplo aUplo, double *aWorkspace, size_t aWorkspaceSize,
                                        size_t aHostSize, size_t aMatrixOrder, double *apMatrix, size_t aLeadingDim,
                                        blas::Layout aLayout, const kernels::RunContext &aContext) {
            // a row-major triangle is the column-major opposite one
            int uplo = Uplo(aUplo);
            if (aLayout == blas::Layout::RowMajor) uplo = uplo == HCGB_UPPER ? HCGB_LOWER : HCGB_UPPER;
            int info = 0;
            Check(hcgb_potrf(aContext.GetHcgbContext(), uplo, I(aMatrixOrder), apMatrix, I(aLeadingDim), &info),
                  aContext, "potrf");
            return info;
        }

        template<>
        void HCoreKernels<double>::FillMatrixTriangle(blas::Uplo aUplo, size_t aRows, size_t aCols,
                                                      double *apMatrix, blas::Layout aLayout, size_t aValue,
                                                      const kernels::RunContext &aContext) {
            if (aRows != aCols) return;
            int uplo = Uplo(aUplo);
            if (aLayout == blas::Layout::RowMajor) uplo = uplo == HCGB_UPPER ? HCGB_LOWER : HCGB_UPPER;
            Check(hcgb_fill_triangle(aContext.GetHcgbContext(), uplo, I(aRows), apMatrix, I(aRows),
                                     static_cast<double>(aValue)), aContext, "FillMatrixTriangle");
        }

        template<>
        void HCoreKernels<double>::trsm(blas::Layout aLayout, blas::Side aSide, blas::Uplo aUplo, blas::Op aTrans,
                                        blas::Diag aDiag, size_t aRows, size_t aCols, double aAlpha,
                                        double const *apMatrixA, size_t aLeadingDimA, double *apMatrixB,
                                        size_t aLeadingDimB, const kernels::RunContext &aContext) {
            ColMajorOnly(aLayout, "trsm");
            Check(hcgb_trsm(aContext.GetHcgbContext(), aSide == blas::Side::Left ? HCGB_LEFT : HCGB_RIGHT,
                            Uplo(aUplo), Trans(aTrans), aDiag == blas::Diag::Unit ? HCGB_UNIT : HCGB_NONUNIT,
                            I(aRows), I(aCols), aAlpha, apMatrixA, I(aLeadingDimA), apMatrixB, I(aLeadingDimB)),
                  aContext, "trsm");
        }

        template<>
        void HCoreKernels<double>::syrk(blas::Layout aLayout, blas::Uplo aUplo, blas::Op aTrans, size_t aRows,
                                        size_t aCols, double aAlpha, double const *apMatrixA, size_t aLeadingDimA,
                                        double aBeta, double *apMatrixB, size_t aLeadingDimB,
                                        const kernels::RunContext &aContext) {
            ColMajorOnly(aLayout, "syrk");
            Check(hcgb_syrk(aContext.GetHcgbContext(), Uplo(aUplo), Trans(aTrans), I(aRows), I(aCols), aAlpha,
                            apMatrixA, I(aLeadingDimA), aBeta, apMatrixB, I(aLeadingDimB)), aContext, "syrk");
        }

        template<>
        void HCoreKernels<double>::Symmetrize(blas::Layout aLayout, double *apMatrixA, size_t aRows, size_t aCols,
                                              blas::Uplo aUplo, const RunContext &aContext) {
            if (aRows != aCols) return;
            int uplo = Uplo(aUplo);
            if (aLayout == blas::Layout::RowMajor) uplo = uplo == HCGB_UPPER ? HCGB_LOWER : HCGB_UPPER;
            Check(hcgb_dsymmetrize(aContext.GetHcgbContext(), uplo, I(aRows), apMatrixA, I(aRows)), aContext,
                  "Symmetrize");
        }

        template<>
        void HCoreKernels<double>::transpose(blas::Layout aLayout, size_t aRows, size_t aCols, const double *aA,
                                             size_t aLeadingDimA, double *aOut, size_t aLeadingDimOut,
                                             const kernels::RunContext &aContext) {
            if (aA == nullptr || aOut == nullptr) return;
            // Out[j + i ldout] = A[i + j lda] for i < min(y, lda), j < min(x, ldout); column-major
            // x = cols, y = rows (row-major: swapped), as src/kernels/omp/kernels.cpp does.
            const size_t x = aLayout == blas::Layout::ColMajor ? aCols : aRows;
            const size_t y = aLayout == blas::Layout::ColMajor ? aRows : aCols;
            const size_t rows = y < aLeadingDimA ? y : aLeadingDimA, cols = x < aLeadingDimOut ? x : aLeadingDimOut;
            Check(hcgb_dcopy2d(aContext.GetHcgbContext(), 1, I(cols), I(rows), 1.0, aA, I(aLeadingDimA), aOut,
                               I(aLeadingDimOut)), aContext, "transpose");
        }

        template<>
        size_t HCoreKernels<double>::CalculatePotrfWorkspaceSize(double *apMatrix, blas::Uplo aUplo,
                                                                 size_t aMatrixOrder, size_t aLeadingDim,
                                                                 size_t &aHostSize, const RunContext &aContext) {
            aHostSize = 0;
            return 0;
        }

        // ------------------------------------------------------------------ float: unsupported
        template<>
        void HCoreKernels<float>::Gemm(blas::Layout, blas::Op, blas::Op, size_t, size_t, size_t, float &,
                                       float const *, size_t, float const *, size_t, float &, float *, size_t,
                                       const RunContext &) { FloatUnsupported("Gemm"); }

        template<>
        void HCoreKernels<float>::MultiplyByAlpha(float *, size_t, size_t, size_t, size_t, float &,
                                                  const RunContext &) { FloatUnsupported("MultiplyByAlpha"); }

        template<>
        void HCoreKernels<float>::ProcessVpointer(size_t, size_t, bool, size_t, float &, float *, size_t, float *,
                                                  size_t, const float *, const RunContext &, bool) {
            FloatUnsupported("ProcessVpointer");
        }

        template<>
        void HCoreKernels<float>::CalculateNewRank(size_t &, bool, float *, size_t, float, const RunContext &) {
            FloatUnsupported("CalculateNewRank");
        }

        template<>
        void HCoreKernels<float>::CalculateUVptr(size_t, size_t, float *, const float *, const RunContext &) {
            FloatUnsupported("CalculateUVptr");
        }

        template<>
        void HCoreKernels<float>::CalculateVTnew(size_t, bool, size_t, float *, float *, size_t, size_t,
                                                 const RunContext &) { FloatUnsupported("CalculateVTnew"); }

        template<>
        void HCoreKernels<float>::CalculateUVptrConj(size_t, size_t, float *, const RunContext &) {
            FloatUnsupported("CalculateUVptrConj");
        }

        template<>
        void HCoreKernels<float>::FillIdentityMatrix(size_t, float *, const RunContext &) {
            FloatUnsupported("FillIdentityMatrix");
        }

        template<>
        void HCoreKernels<float>::LaCpy(common::MatrixType, size_t, size_t, float *, size_t, float *, size_t,
                                        const RunContext &) { FloatUnsupported("LaCpy"); }

        template<>
        void HCoreKernels<float>::Geqrf(size_t, size_t, float *, size_t, float *, float *, size_t, size_t,
                                        const RunContext &) { FloatUnsupported("Geqrf"); }

        template<>
        void HCoreKernels<float>::Laset(common::MatrixType, size_t, size_t, float, float, float *, size_t,
                                        const RunContext &) { FloatUnsupported("Laset"); }

        template<>
        void HCoreKernels<float>::Trmm(blas::Layout, blas::Side, blas::Uplo, blas::Op, blas::Diag, size_t, size_t,
                                       float, float const *, size_t, float *, size_t, const RunContext &) {
            FloatUnsupported("Trmm");
        }

        template<>
        void HCoreKernels<float>::SVD(common::Job, common::Job, size_t, size_t, float *, size_t, float *, float *,
                                      size_t, float *, size_t, common::CompressionType, float *, size_t, size_t,
                                      const RunContext &) { FloatUnsupported("SVD"); }

        template<>
        void HCoreKernels<float>::Unmqr(common::SideMode, common::BlasOperation, size_t, size_t, size_t,
                                        float const *, size_t, float const *, float *, size_t, float *, size_t,
                                        const RunContext &) { FloatUnsupported("Unmqr"); }

        template<>
        void HCoreKernels<float>::ungqr(size_t, size_t, size_t, float *, size_t, float *, float *, size_t,
                                        const RunContext &) { FloatUnsupported("ungqr"); }

        template<>
        size_t HCoreKernels<float>::CalculateGemmWorkspaceSize(size_t, size_t, size_t, size_t, size_t,
                                                               const operators::CompressionParameters &, size_t &,
                                                               const RunContext &) {
            FloatUnsupported("CalculateGemmWorkspaceSize");
        }

        template<>
        int HCoreKernels<float>::potrf(blas::Uplo, float *, size_t, size_t, size_t, float *, size_t, blas::Layout,
                                       const kernels::RunContext &) { FloatUnsupported("potrf"); }

        template<>
        void HCoreKernels<float>::FillMatrixTriangle(blas::Uplo, size_t, size_t, float *, blas::Layout, size_t,
                                                     const kernels::RunContext &) {
            FloatUnsupported("FillMatrixTriangle");
        }

        template<>
        void HCoreKernels<float>::trsm(blas::Layout, blas::Side, blas::Uplo, blas::Op, blas::Diag, size_t, size_t,
                                       float, float const *, size_t, float *, size_t, const kernels::RunContext &) {
            FloatUnsupported("trsm");
        }

        template<>
        void HCoreKernels<float>::syrk(blas::Layout, blas::Uplo, blas::Op, size_t, size_t, float, float const *,
                                       size_t, float, float *, size_t, const kernels::RunContext &) {
            FloatUnsupported("syrk");
        }

        template<>
        void HCoreKernels<float>::Symmetrize(blas::Layout, float *, size_t, size_t, blas::Uplo, const RunContext &) {
            FloatUnsupported("Symmetrize");
        }

        template<>
        void HCoreKernels<float>::transpose(blas::Layout, size_t, size_t, const float *, size_t, float *, size_t,
                                            const kernels::RunContext &) { FloatUnsupported("transpose"); }

        template<>
        size_t HCoreKernels<float>::CalculatePotrfWorkspaceSize(float *, blas::Uplo, size_t, size_t, size_t &,
                                                                const RunContext &) {
            FloatUnsupported("CalculatePotrfWorkspaceSize");
        }
    }
}
