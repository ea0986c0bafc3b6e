// Shared pieces of the command-line drivers: each driver keeps the command
// line and the printed checksums of the reference app it replaces
// (src/apps/graph_analytics/*.cpp, src/apps/information_retrieval/bm25.cpp)
// and runs it through the C ABI in la3g.h.
#ifndef LA3G_DRIVER_COMMON_H
#define LA3G_DRIVER_COMMON_H

#include <cstdint>
#include <string>
#include <vector>

#include "la3g.h"

// Exits with the library's message when st is not LA3G_OK.
void check(int st, const char* what);
// Loads path with flags (n = 0: the vertex count comes from the file header).
la3g_graph* load(const char* path, uint32_t n, uint32_t flags, uint32_t nright = 0);
uint32_t nslots(la3g_graph* g);
// Prints "<name>: <ms> ms (device <ms> ms)" from a call's stats.
void report(const char* name, const la3g_stats& st);
// prepare_queries (information_retrieval/helpers.hpp:76-123): label i of the
// term labels file is vertex terms_offset + i + 1; unknown labels map to 0.
std::vector<std::vector<uint32_t>> read_queries(const std::string& labels, const std::string& queries,
                                                uint32_t terms_offset);

#endif
