// stubs.cu — temporary: entry points not implemented yet.
#include "index.cuh"
using namespace gn;
extern "C" {
int gn_kmeans_l2(const float *, int64_t, int64_t, int64_t, int64_t, uint32_t, int32_t *, float *, int64_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_create(int32_t, int32_t, gn_index **) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_set(gn_index *, const float *, int64_t, int64_t) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_set_assigned(gn_index *, const float *, int64_t, int64_t, const float *, int32_t, const int32_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_search_knn(gn_index *, const float *, int64_t, int64_t, int64_t *, float *, int64_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_search_knn_device(gn_index *, const float *, int64_t, int64_t, int64_t *, float *, int64_t *, void *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_set_n_probe(gn_index *, int32_t) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_info(gn_index *, int32_t *, int32_t *, int64_t *, int64_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfl2_export(gn_index *, float *, int64_t *, int64_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfbin_create(int32_t, int32_t, int32_t, uint32_t, gn_index **) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfbin_set(gn_index *, const uint8_t *, int64_t, int64_t) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfbin_search_knn(gn_index *, const uint8_t *, int64_t, int64_t, int64_t *, int64_t *, int64_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfbin_get_params(gn_index *, int32_t *, int32_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfbin_set_nprobe(gn_index *, int32_t) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
int gn_ivfbin_export(gn_index *, uint8_t *, int32_t *, int32_t *) { return fail(GN_ERR_UNSUPPORTED, "not yet"); }
}
