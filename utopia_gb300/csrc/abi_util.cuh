// Helpers shared by the C-ABI entry points: exception -> status code translation.
#pragma once
#include "internal.cuh"

namespace ugpu {
extern thread_local std::string g_last_error;

inline void set_error(Context *ctx, const char *msg) {
    g_last_error = msg;
    if (ctx) ctx->last_error = msg;
}
}  // namespace ugpu

#define UGPU_ABI_BEGIN try {
#define UGPU_ABI_END(ctxptr)                                              \
    }                                                                     \
    catch (const ::ugpu::Error &e) {                                      \
        ::ugpu::set_error((ctxptr), e.what());                            \
        return e.code;                                                    \
    }                                                                     \
    catch (const std::bad_alloc &e) {                                     \
        ::ugpu::set_error((ctxptr), "host allocation failed");            \
        return UGPU_ERR_ALLOC;                                            \
    }                                                                     \
    catch (const std::exception &e) {                                     \
        ::ugpu::set_error((ctxptr), e.what());                            \
        return UGPU_ERR_INTERNAL;                                         \
    }                                                                     \
    return UGPU_OK;

#define UGPU_REQUIRE(ptr) UGPU_CHECK((ptr) != nullptr, UGPU_ERR_ARG, "null handle: " #ptr)
