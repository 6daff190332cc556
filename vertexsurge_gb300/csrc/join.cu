// Vertex-id hash join (placeholder, replaced below).
#include "vs_internal.cuh"
using namespace vs;
extern "C" int vs_hash_join(vs_table_ref a, vs_table_ref b, int only_count, uint64_t max_rows,
                            vs_flat **out, uint64_t *count, vs_stream_t stream) {
  (void)a; (void)b; (void)only_count; (void)max_rows; (void)out; (void)count; (void)stream;
  return fail(VS_ERR_UNSUPPORTED, "vs_hash_join not built yet");
}
