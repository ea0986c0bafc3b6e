// graphsim <data_graph_labels> <data_graph_matrix> <nvertices> <query_graph_labels> <query_graph_matrix>
// (src/apps/graph_simulation/graphsim.cpp:45-119): graph simulation of a
// query graph on the data graph, run by the vertex program in
// libla3g_programs.so.  Inputs are read by the reference's rules: data labels
// one {"key":"label"} line per vertex after a "[" line (a first line "null,"
// leaves vertex 0 unlabelled); query labels as whitespace-separated tokens
// read until end of file (a file ending in whitespace adds an empty label);
// the query matrix as "i j" pairs.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "driver_common.h"
#include "la3g_programs.h"

static std::vector<std::string> read_data_labels(const char* path, uint32_t n)
{
  std::vector<std::string> labels(n);
  std::ifstream f(path);
  if (!f.good())
  {
    std::fprintf(stderr, "Could not read file %s \n", path);
    std::exit(1);
  }
  char buf[2048];
  f.getline(buf, sizeof buf);  // "["
  for (uint32_t i = 0; i < n; i++)
  {
    f.getline(buf, sizeof buf);
    if (i == 0 && std::strcmp(buf, "null,") == 0) continue;
    char* t = std::strtok(buf, ":");
    t = t ? std::strtok(nullptr, ":") : nullptr;
    t = t ? std::strtok(t + 1, "\"") : nullptr;
    if (t) labels[i] = t;
  }
  return labels;
}

static std::vector<std::string> read_query_labels(const char* path)
{
  std::vector<std::string> labels;
  std::ifstream f(path);
  while (!f.eof())
  {
    std::string l;
    f >> l;
    labels.push_back(l);
  }
  return labels;
}

static std::vector<uint32_t> read_query_edges(const char* path)
{
  std::vector<uint32_t> e;
  std::ifstream f(path);
  while (!f.eof())
  {
    int i = 0, j = 0;
    f >> i;
    if (f.eof()) break;
    f >> j;
    e.push_back((uint32_t) i);
    e.push_back((uint32_t) j);
  }
  return e;
}

int main(int argc, char** argv)
{
  if (argc < 6)
  {
    std::printf("Usage: %s <data_graph_labels_filepath> <data_graph_matrix_filepath> <nvertices> "
                "<query_graph_labels_filepath> <query_graph_matrix_filepath> \n",
                argv[0]);
    return 1;
  }
  const uint32_t n = (uint32_t) std::atoi(argv[3]);
  la3g_graph* g = load(argv[2], n, LA3G_DIRECTED | LA3G_REVERSE);
  const uint32_t N = nslots(g);
  const std::vector<std::string> dl = read_data_labels(argv[1], n);
  const std::vector<std::string> ql = read_query_labels(argv[4]);
  const std::vector<uint32_t> qe = read_query_edges(argv[5]);
  std::unordered_map<std::string, uint32_t> ids{{"", 0}};
  auto lid = [&](const std::string& s) { return ids.emplace(s, (uint32_t) ids.size()).first->second; };
  std::vector<uint32_t> vlabel(N, 0), qlabel;
  for (uint32_t v = 0; v < n && v < N; v++) vlabel[v] = lid(dl[v]);
  for (const auto& s : ql) qlabel.push_back(lid(s));
  std::vector<uint8_t> matched(N);
  uint32_t nm = 0, iters = 0;
  check(la3gp_graphsim(g, vlabel.data(), (uint32_t) qlabel.size(), qlabel.data(), qe.data(),
                       (uint32_t) (qe.size() / 2), matched.data(), nullptr, &nm, &iters),
        "graphsim");
  for (uint32_t v = 0; v < N && v <= n; v++)
  {
    if (matched[v]) std::printf("%u: %u\n", v, v);
    else std::printf("%u: \n", v);
  }
  std::printf("Num matches = %u \n", nm);
  std::printf("Iterations = %u \n", iters);
  la3g_graph_free(g);
  return 0;
}
