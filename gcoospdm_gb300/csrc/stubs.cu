// temporary: batch and autotune not yet built
#include "handle.hpp"
namespace gcoo {
bool tuned_params(int64_t, int64_t, int64_t, int64_t, gcoo_params *) { return false; }
}
extern "C" {
gcoo_status gcoo_batch_create(gcoo_batch **, const gcoo_problem *, int32_t, gcoo_precision, void *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_batch_run(gcoo_batch *, void *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_batch_launches(const gcoo_batch *, int32_t *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_batch_destroy(gcoo_batch *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_autotune(gcoo_handle *, const float *, int64_t, float *, void *, gcoo_params *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_autotune_save(const char *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_autotune_load(const char *) { return GCOO_ERROR_UNSUPPORTED; }
gcoo_status gcoo_autotune_clear(void) { return GCOO_ERROR_UNSUPPORTED; }
}
