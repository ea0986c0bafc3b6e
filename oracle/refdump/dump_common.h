/*
 * Helpers shared by the reference dump drivers.  These drivers are test
 * infrastructure: each one includes an LA3 app header from the reference,
 * replays that app's run() sequence call for call, and writes every
 * per-vertex result (indexed by original vertex id) to a binary file so that
 * the oracle restatement and the GPU path can be compared against the
 * reference itself.  One JSON line with the execution time (the window the
 * app's own DistTimer measures) and the app's checksums goes to stdout.
 */
#ifndef LA3_REFDUMP_COMMON_H
#define LA3_REFDUMP_COMMON_H
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

template <class T>
static void dump_array(const std::string& path, const std::vector<T>& v)
{
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (!v.empty() && std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size())
  { std::perror(path.c_str()); std::exit(2); }
  std::fclose(f);
}
#endif
