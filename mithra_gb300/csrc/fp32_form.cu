// Mixed-precision form: placeholder entry points until the FP32 kernels are in place.
#include "ctx.h"

namespace mithra {
int fp32_alloc(mithra_ctx* ctx) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
void fp32_free(mithra_ctx*) {}
float* fp32_field(mithra_ctx* ctx, int level) { return ctx->f32.A[ctx->idx[level]]; }
float* fp32_scalar(mithra_ctx* ctx, int level) { return ctx->f32.F[ctx->idx[level]]; }
int fp32_records_to_soa(mithra_ctx* ctx, const double*, long long) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_soa_to_records(mithra_ctx* ctx, double*, long long, long long*) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_field_update(mithra_ctx* ctx) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_eval_eb(mithra_ctx* ctx) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_push(mithra_ctx* ctx, int) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_save_positions(mithra_ctx* ctx) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_erase(mithra_ctx* ctx) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
int fp32_current(mithra_ctx* ctx) { return fail(ctx, MITHRA_ERR_ARG, "FP32 form not available"); }
}  // namespace mithra
