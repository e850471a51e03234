/*
 * kernels::RunContext of the GB300 backend (declared in include/hcorepp/kernels/gb300/RunContext.hpp),
 * on libhcgb's C ABI.  Replaces src/kernels/cuda/RunContext.cpp for a USE_GB300 build.
 */
#include <hcorepp/kernels/RunContext.hpp>

#include <stdexcept>
#include <string>

namespace hcorepp {
    namespace kernels {
        struct RunContext::State {
            int device = 0;
            cudaStream_t stream = nullptr;
            hcgb_context *ctx = nullptr;
            int *info = nullptr;
            void *work = nullptr;
            size_t work_bytes = 0;

            ~State() {
                if (ctx) hcgb_context_destroy(ctx);
                if (stream) {
                    cudaStreamSynchronize(stream);
                    cudaStreamDestroy(stream);
                }
                if (info) cudaFree(info);
                if (work) cudaFree(work);
            }
        };

        namespace {
            void Check(cudaError_t aError, const char *apWhat) {
                if (aError != cudaSuccess) {
                    throw std::runtime_error(std::string(apWhat) + ": " + cudaGetErrorString(aError));
                }
            }
        }

        RunContext::RunContext() : mpState(std::make_shared<State>()) {
            Check(cudaGetDevice(&mpState->device), "RunContext");
            Check(cudaStreamCreateWithFlags(&mpState->stream, cudaStreamNonBlocking), "RunContext");
            if (hcgb_context_create(mpState->device, mpState->stream, &mpState->ctx) != HCGB_OK) {
                throw std::runtime_error("RunContext: hcgb_context_create failed");
            }
            Check(cudaMalloc((void **) &mpState->info, sizeof(int)), "RunContext");
        }

        RunContext::RunContext(const RunContext &aContext) = default;

        RunContext &RunContext::operator=(const RunContext &aContext) = default;

        cudaStream_t RunContext::GetStream() const {
            return mpState->stream;
        }

        hcgb_context *RunContext::GetHcgbContext() const {
            return mpState->ctx;
        }

        int *RunContext::GetInfoPointer() const {
            return mpState->info;
        }

        void *RunContext::RequestWorkBuffer(size_t aBufferSize) const {
            if (aBufferSize > mpState->work_bytes) {
                if (mpState->work) {
                    Check(cudaStreamSynchronize(mpState->stream), "RequestWorkBuffer");
                    Check(cudaFree(mpState->work), "RequestWorkBuffer");
                    mpState->work = nullptr;
                }
                Check(cudaMalloc(&mpState->work, aBufferSize), "RequestWorkBuffer");
                mpState->work_bytes = aBufferSize;
            }
            return mpState->work;
        }

        void RunContext::Sync() const {
            if (hcgb_sync(mpState->ctx) != HCGB_OK) {
                throw std::runtime_error(std::string("RunContext::Sync: ") + hcgb_last_error(mpState->ctx));
            }
        }

        RunContext RunContext::ForkChildContext() {
            return RunContext();
        }

        RunContext::~RunContext() = default;
    }//namespace kernels
}//namespace hcorepp
