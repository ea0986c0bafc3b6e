// la3g_gen: writes the seeded synthetic inputs of this library as LA3 binary
// edge files, from the generator sources alone (host C++; no CUDA and no
// libla3g), so that a CPU-only consumer - for instance the reference's own
// apps timed as a baseline - reads exactly the records the library's
// EdgeList generators produce for the same arguments.
//
//   la3g_gen rmat <scale> <edge_factor> <seed> <out> [wseed]
//   la3g_gen er   <n> <m0> <seed> <out> [wseed]
//
// R-MAT uses a, b, c = 0.57, 0.19, 0.19; a trailing wseed writes u32-weighted
// triples (weights uniform in [1, 128]) instead of pairs.  Records carry
// 1-based ids, self-loops and duplicates removed, no header.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "la3g.h"
#include "la3g_internal.h"

namespace la3g {

static char g_msg[1024];

int set_error(int code, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_msg, sizeof g_msg, fmt, ap);
  va_end(ap);
  return code;
}

}  // namespace la3g

static int usage()
{
  std::fprintf(stderr,
               "usage: la3g_gen rmat <scale> <edge_factor> <seed> <out> [wseed]\n"
               "       la3g_gen er <n> <m0> <seed> <out> [wseed]\n");
  return 1;
}

int main(int argc, char** argv)
{
  if (argc < 6) return usage();
  const std::string kind = argv[1];
  const unsigned long long a1 = std::strtoull(argv[2], nullptr, 10), a2 = std::strtoull(argv[3], nullptr, 10),
                           seed = std::strtoull(argv[4], nullptr, 10);
  const char* out = argv[5];
  const bool weighted = argc > 6;
  const unsigned long long wseed = weighted ? std::strtoull(argv[6], nullptr, 10) : 0;
  la3g_edges e;
  int rc;
  if (kind == "rmat")
    rc = la3g_gen_rmat((uint32_t) a1, (uint32_t) a2, 0.57, 0.19, 0.19, seed, weighted ? 1 : 0, wseed, &e);
  else if (kind == "er")
    rc = la3g_gen_er((uint32_t) a1, a2, seed, weighted ? 1 : 0, wseed, &e);
  else
    return usage();
  if (rc == LA3G_OK) rc = la3g_edges_write(&e, out, 0);
  if (rc != LA3G_OK)
  {
    std::fprintf(stderr, "la3g_gen: %s\n", la3g::g_msg);
    la3g_edges_free(&e);
    return 2;
  }
  std::printf("{\"n\": %u, \"m\": %llu, \"weighted\": %d}\n", e.n, (unsigned long long) e.m, weighted ? 1 : 0);
  la3g_edges_free(&e);
  return 0;
}
