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
int kf_mlp_create(int32_t, int32_t, int32_t, uint64_t, kf_mlp **) { return pending("kf_mlp_create"); }
int kf_mlp_destroy(kf_mlp *) { return pending("kf_mlp_destroy"); }
int kf_mlp_set_scaling(kf_mlp *, const float *, const float *, const float *, const float *) {
    return pending("kf_mlp_set_scaling");
}
int kf_mlp_train(kf_mlp *, const float *, const float *, int64_t, int32_t, int32_t, float, uint64_t, float *) {
    return pending("kf_mlp_train");
}
int kf_mlp_forward(kf_mlp *, const float *, float *, int64_t) { return pending("kf_mlp_forward"); }
int kf_mlp_gradients(kf_mlp *, const float *, const float *, int64_t, float *, float *) {
    return pending("kf_mlp_gradients");
}
int kf_mlp_get_params(kf_mlp *, float *, int64_t *) { return pending("kf_mlp_get_params"); }
}
