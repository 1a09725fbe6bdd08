// Entry points whose kernels are not in this build yet: they fail loudly with KF_EINVAL.
#include "kf_internal.h"

extern "C" {
static int pending(const char *what) {
    kf::set_last_error(std::string(what) + ": not available in this build");
    return KF_EINVAL;
}
int kf_batch_solve(const kf_op_desc *, int32_t, const int32_t *, double, int32_t, int32_t, double *, double *,
                   int32_t *, double *) { return pending("kf_batch_solve"); }
int kf_batch_autotune(const kf_op_desc *, int32_t, const int32_t *, double, int32_t, int32_t *) {
    return pending("kf_batch_autotune");
}
}
