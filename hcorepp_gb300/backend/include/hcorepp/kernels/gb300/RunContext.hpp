/*
 * GB300 backend of HCore++'s kernels::RunContext (the role of
 * include/hcorepp/kernels/cuda/RunContext.hpp:15-53): one device, one CUDA stream and one
 * libhcgb context (include/hcgb.h) whose grow-only device workspace serves RequestWorkBuffer.
 * Selected in the reference's include/hcorepp/kernels/RunContext.hpp by USE_GB300.
 */
#ifndef HCOREPP_KERNELS_GB300_RUN_CONTEXT_HPP
#define HCOREPP_KERNELS_GB300_RUN_CONTEXT_HPP

#include <cuda_runtime.h>

#include <cstddef>
#include <memory>

#include "hcgb.h"

namespace hcorepp {
    namespace kernels {
        class RunContext {
        public:
            /** A new stream (non-blocking) and libhcgb context on the current device. */
            RunContext();

            /** Shares the stream and libhcgb context of aContext, as the CUDA backend's copy shares its handles. */
            RunContext(const RunContext &aContext);

            RunContext &operator=(const RunContext &aContext);

            cudaStream_t GetStream() const;

            /** The libhcgb context the kernels of this backend run on. */
            hcgb_context *GetHcgbContext() const;

            /** A device int for status words (potrf info). */
            int *GetInfoPointer() const;

            /** Device scratch of at least aBufferSize bytes, owned by the context, valid until the next call. */
            void *RequestWorkBuffer(size_t aBufferSize) const;

            void Sync() const;

            /** A context on a new stream of the same device (its own libhcgb context). */
            RunContext ForkChildContext();

            ~RunContext();

            bool SupportsOMP() const {
                return false;
            }

        private:
            struct State;
            std::shared_ptr<State> mpState;
        };
    }//namespace kernels
}//namespace hcorepp

#endif //HCOREPP_KERNELS_GB300_RUN_CONTEXT_HPP
