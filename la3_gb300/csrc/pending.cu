// Entry points whose device implementation is not in this build yet; each
// returns LA3G_EINVAL with a message naming itself.
#include "la3g_internal.h"

using namespace la3g;

extern "C" int la3g_bfs_batch(la3g_graph*, const uint32_t*, uint32_t, uint8_t*, la3g_stats*)
{
  return set_error(LA3G_EINVAL, "la3g_bfs_batch is not available in this build");
}

extern "C" int la3g_sssp_batch(la3g_graph*, const uint32_t*, uint32_t, uint32_t*, la3g_stats*)
{
  return set_error(LA3G_EINVAL, "la3g_sssp_batch is not available in this build");
}
