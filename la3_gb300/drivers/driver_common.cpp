#include "driver_common.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <unordered_map>

void check(int st, const char* what)
{
  if (st == LA3G_OK) return;
  std::fprintf(stderr, "%s failed: %s (%s)\n", what, la3g_status_string(st), la3g_last_error_string());
  std::exit(1);
}

la3g_graph* load(const char* path, uint32_t n, uint32_t flags, uint32_t nright)
{
  la3g_graph* g = nullptr;
  check(la3g_graph_load(path, n, nright, flags, &g), "load");
  return g;
}

uint32_t nslots(la3g_graph* g)
{
  la3g_graph_info gi;
  check(la3g_graph_info_get(g, &gi), "info");
  return gi.nslots;
}

void report(const char* name, const la3g_stats& st)
{
  std::printf("%s: %.3f ms (device %.3f ms)\n", name, st.host_ms, st.device_ms);
}

std::vector<std::vector<uint32_t>> read_queries(const std::string& labels, const std::string& queries,
                                                uint32_t terms_offset)
{
  std::unordered_map<std::string, uint32_t> id;
  std::ifstream fl(labels);
  if (!fl) check(LA3G_EIO, labels.c_str());
  std::string line;
  uint32_t i = 0;
  while (std::getline(fl, line))
  {
    std::istringstream ss(line);
    std::string label;
    if (!(ss >> label)) continue;
    id[label] = terms_offset + i + 1;
    i++;
  }
  std::ifstream fq(queries);
  if (!fq) check(LA3G_EIO, queries.c_str());
  std::vector<std::vector<uint32_t>> out;
  while (std::getline(fq, line))
  {
    std::istringstream ss(line);
    std::vector<uint32_t> q;
    std::string t;
    while (ss >> t)
    {
      auto it = id.find(t);
      q.push_back(it == id.end() ? 0u : it->second);
    }
    if (!q.empty()) out.push_back(q);
  }
  return out;
}
