// split_api.h — host interface of the tensor-core forms (split-precision, BF16x3, BF16).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "gb300_internal.h"

namespace gb {

struct SplitRequest {
    int method = 0;            // gb300_method (AUTO, NATIVE, SPLIT, BF16X3 or BF16)
    int slices = 0;            // slices per operand; 0 = choose from target_error
    double target_error = 0;   // normwise target; <= 0 means k * 2^-53
    int max_sms = 0;           // cap on the persistent tensor-core grid (0: every SM)
};

struct SplitResult {
    int method_used = 0;
    int slices = 0;
    double error_bound = 0;
    const void* info_dev = nullptr;  // device copy of the slice count and bound (tensor-core forms)
};

// Read the slice count and the a-priori bound back from the device copy (after the stream has
// finished the product).
bool split_read_info(const void* info_dev, int* slices, double* bound);
// Size of the device record split_read_info reads, and its decoding from a host copy (the serving
// loop copies it back asynchronously behind the product).
size_t split_info_bytes();
void split_decode_info(const void* info_host, int* slices, double* bound);

struct Workspace;

// Runs the double-precision product g (operands on the device, TMA-aligned) with the requested
// form on stream `s`, taking scratch from `ws`.  AUTO picks between the split form and the native
// kernel.  Returns a gb300_status.
int device_product(const Gemm& g, const SplitRequest& req, const LaunchCtl& ctl, cudaStream_t s, Workspace& ws,
                   SplitResult* out, std::string* err);

// True when the `auto` method runs a product on the native kernel (small products, short k).
bool split_auto_uses_native(const Gemm& g);

// The same for float operands (device, float, caller's pitches): widened to double in `conv`
// (slots 0-2), computed at the float target k 2^-24 unless the request sets one, rounded once to
// float.  The bound includes the final rounding (2^-24).
int device_product_float(const Gemm& g, const SplitRequest& req, const LaunchCtl& ctl, cudaStream_t s, Workspace& ws,
                         Workspace& conv, SplitResult* out, std::string* err);

// FP64-accurate product of host operands (page-locked or pageable) in row panels of A: B is copied
// and sliced once, then each panel's copy in, product and copy of C back run on three streams so
// that the transfers overlap the computation.  The operands keep the caller's layout (g as for device_product, with host
// pointers); the call's work ends on stream s.  Returns GB300_ERR_NOT_SUPPORTED, with nothing
// enqueued, when the method or shape does not qualify: the caller then stages the operands
// and calls device_product.
int device_product_host_panels(const Gemm& g, const SplitRequest& req, const LaunchCtl& ctl, cudaStream_t s,
                               Workspace& ws, SplitResult* out, std::string* err);

// Device scratch bytes device_product needs for g (admission control): per workspace slot, rounded
// the way Workspace::get rounds, and their sum.
void device_product_slot_needs(const Gemm& g, const SplitRequest& req, size_t need[]);
size_t device_product_footprint(const Gemm& g, const SplitRequest& req);

}  // namespace gb
