// Multi-way intersection (placeholder, replaced below).
#include "vs_internal.cuh"
using namespace vs;
extern "C" int vs_mintersect(vs_table_ref base, const vs_isect_dep *deps, uint32_t ndeps,
                             uint32_t new_vertex_count, int only_count, uint64_t max_rows,
                             vs_flat **out, uint64_t *count, vs_stream_t stream) {
  (void)base; (void)deps; (void)ndeps; (void)new_vertex_count; (void)only_count; (void)max_rows;
  (void)out; (void)count; (void)stream;
  return fail(VS_ERR_UNSUPPORTED, "vs_mintersect not built yet");
}
