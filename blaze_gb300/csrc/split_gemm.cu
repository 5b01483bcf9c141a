// split_gemm.cu — tensor-core forms of the double-precision product (placeholder: AUTO runs the
// native kernel; the explicit tensor-core methods report that they are not built yet).
#include "../../include/gb300_blas.h"
#include "runtime.h"
#include "split_api.h"

namespace gb {

int split_gemm(const Gemm& g, const SplitRequest& req, const LaunchCtl& ctl, cudaStream_t s, SplitResult* out,
               std::string* err) {
    if (req.method != GB300_METHOD_AUTO) {
        if (err) *err = "tensor-core forms are not available in this build";
        return GB300_ERR_NOT_SUPPORTED;
    }
    Runtime& r = runtime();
    int splits = native_choose_splits(g.m, g.n, g.k, 8, r.num_sms);
    double* ws = nullptr;
    if (splits > 1) {
        ws = static_cast<double*>(pool_get(kSlotWork, size_t(splits) * size_t(g.m) * size_t(g.n) * 8, err));
        if (!ws) return GB300_ERR_NO_MEMORY;
    }
    cudaError_t e = native_gemm<double>(g, splits, ws, ctl, s, err);
    if (e != cudaSuccess) return GB300_ERR_CUDA;
    out->method_used = GB300_METHOD_NATIVE;
    out->slices = 0;
    out->error_bound = double(g.k) * 0x1p-53;
    return GB300_OK;
}

}  // namespace gb
