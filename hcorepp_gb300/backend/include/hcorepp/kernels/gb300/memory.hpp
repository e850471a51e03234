/*
 * GB300 backend of HCore++'s memory abstraction (the role of include/hcorepp/kernels/cuda/memory.hpp:
 * every tile buffer is device memory): allocation, release, copies and memset on the context stream.
 * Errors throw std::runtime_error (the CUDA backend exits through GPU_ERROR_CHECK).
 */
#ifndef HCOREPP_KERNELS_GB300_MEMORY_HPP
#define HCOREPP_KERNELS_GB300_MEMORY_HPP

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

namespace hcorepp {
    namespace memory {
        namespace gb300_detail {
            inline void check(cudaError_t aError, const char *apWhat) {
                if (aError != cudaSuccess) {
                    throw std::runtime_error(std::string(apWhat) + ": " + cudaGetErrorString(aError));
                }
            }
        }

        template<typename T>
        T *AllocateArray(size_t aNumElements, const hcorepp::kernels::RunContext &aContext) {
            T *array = nullptr;
            gb300_detail::check(cudaMalloc((void **) &array, aNumElements * sizeof(T)), "AllocateArray");
            return array;
        }

        template<typename T>
        void DestroyArray(T *apArray, const hcorepp::kernels::RunContext &aContext) {
            if (apArray != nullptr) {
                gb300_detail::check(cudaFree(apArray), "DestroyArray");
            }
        }

        template<typename T>
        void Memcpy(T *apDestination, const T *apSrcDataArray, size_t aNumOfElements,
                    const hcorepp::kernels::RunContext &aContext, MemoryTransfer aTransferType, bool aBlocking) {
            gb300_detail::check(cudaMemcpyAsync(apDestination, apSrcDataArray, aNumOfElements * sizeof(T),
                                                cudaMemcpyDefault, aContext.GetStream()), "Memcpy");
            if (aBlocking) {
                gb300_detail::check(cudaStreamSynchronize(aContext.GetStream()), "Memcpy");
            }
        }

        template<typename T>
        void Memset(T *apDestination, char aValue, size_t aNumOfElements,
                    const hcorepp::kernels::RunContext &aContext) {
            gb300_detail::check(cudaMemsetAsync(apDestination, aValue, aNumOfElements * sizeof(T),
                                                aContext.GetStream()), "Memset");
        }

        template<typename T>
        T *Realloc(T *apDataArray, size_t aNumOfElements, const hcorepp::kernels::RunContext &aContext) {
            DestroyArray(apDataArray, aContext);
            return AllocateArray<T>(aNumOfElements, aContext);
        }
    }//namespace memory
}//namespace hcorepp

#endif //HCOREPP_KERNELS_GB300_MEMORY_HPP
