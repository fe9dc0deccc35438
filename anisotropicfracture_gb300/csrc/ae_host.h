// Host-side error plumbing shared by the C-ABI translation units: an exception per failure,
// mapped to an ae_status (and a message for ae_last_error) at the ABI boundary.
#pragma once
#include <cuda_runtime.h>

#include <new>
#include <stdexcept>
#include <string>

#include "../../include/aefast.h"
#include "ae_launch.h"

namespace ae {
namespace hx {

struct ApiErr : std::runtime_error {
    int code;
    ApiErr(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
struct CudaErr : std::runtime_error {
    cudaError_t err;
    CudaErr(const std::string& m, cudaError_t e) : std::runtime_error(m), err(e) {}
};

#define AEH_CHECK(x)                                                                                \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess)                                                                      \
            throw ::ae::hx::CudaErr(std::string(cudaGetErrorString(e_)) + " at " + __FILE__ + ":" + \
                                        std::to_string(__LINE__),                                   \
                                    e_);                                                            \
    } while (0)

template <class F>
int guarded(F&& f) {
    try {
        f();
        return AE_OK;
    } catch (const ApiErr& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const CudaErr& e) {
        set_last_error(e.what());
        return e.err == cudaErrorMemoryAllocation ? AE_ERR_OOM : AE_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return AE_ERR_OOM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return (std::string(e.what()).find("out of memory") != std::string::npos) ? AE_ERR_OOM : AE_ERR_CUDA;
    }
}

inline void require(bool ok, const std::string& msg, int code = AE_ERR_ARG) {
    if (!ok) throw ApiErr(code, msg);
}

inline bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace hx
}  // namespace ae
