/*
 * la3_oracle command-line tool (test infrastructure only).
 *
 *   la3_oracle pr   <file> <n> <iters> <out_prefix>
 *   la3_oracle bfs  <file> <n> <root> <out_prefix>
 *   la3_oracle sssp <file.w> <n> <root> <out_prefix>
 *   la3_oracle cc   <file> <n> <out_prefix>
 *   la3_oracle tc   <file> <n> <out_prefix>
 *
 * Writes the same per-vertex files as the reference dump drivers
 * (<out_prefix>.rank.f64, .hops.u8, .parent.u32, .dist.u32, .label.u32,
 * .ntri.u32) and one JSON line with the execution time and checksums; the
 * timed window excludes ingest, like the apps' own DistTimer windows.
 */
#define _POSIX_C_SOURCE 199309L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "la3_oracle.h"

static double now(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

static void dump(const char* prefix, const char* suffix, const void* p, size_t bytes)
{
  char path[4096];
  snprintf(path, sizeof path, "%s%s", prefix, suffix);
  FILE* f = fopen(path, "wb");
  if (!f || fwrite(p, 1, bytes, f) != bytes) { perror(path); exit(2); }
  fclose(f);
}

static og_graph* load(const char* path, uint32_t n, uint32_t flags)
{
  og_graph* g = NULL;
  int rc = og_load(path, n, 0, flags, &g);
  if (rc) { fprintf(stderr, "la3_oracle: %s\n", og_last_error()); exit(1); }
  return g;
}

int main(int argc, char** argv)
{
  if (argc < 5) { fprintf(stderr, "usage: la3_oracle <app> <file> <n> [arg] <out_prefix>\n"); return 1; }
  const char* app = argv[1];
  const char* path = argv[2];
  uint32_t n = (uint32_t) strtoul(argv[3], NULL, 10);
  if (!strcmp(app, "pr") || !strcmp(app, "bfs") || !strcmp(app, "sssp"))
  {
    if (argc < 6) { fprintf(stderr, "missing argument\n"); return 1; }
    uint32_t arg = (uint32_t) strtoul(argv[4], NULL, 10);
    const char* out = argv[5];
    if (!strcmp(app, "pr"))
    {
      og_graph* g = load(path, n, OG_DIRECTED);
      uint32_t N = og_nslots(g);
      double* rank = malloc(N * sizeof(double));
      uint32_t* deg = malloc(N * sizeof(uint32_t));
      double t0 = now();
      og_pagerank(g, arg, rank, deg);
      double t = now() - t0;
      long dsum = 0; double rsum = 0;
      for (uint32_t i = 0; i < N; i++) { dsum += deg[i]; rsum += rank[i]; }
      dump(out, ".rank.f64", rank, N * sizeof(double));
      dump(out, ".degree.u32", deg, N * sizeof(uint32_t));
      printf("{\"app\": \"pr\", \"exec_s\": %.9f, \"degree_checksum\": %ld, \"pr_checksum\": %.17g, "
             "\"nslots\": %u, \"nedges\": %llu}\n", t, dsum, rsum, N, (unsigned long long) og_nedges(g));
      og_free(g);
    }
    else if (!strcmp(app, "bfs"))
    {
      og_graph* g = load(path, n, 0);
      uint32_t N = og_nslots(g), it = 0;
      uint8_t* hops = malloc(N);
      uint32_t* parent = malloc(N * sizeof(uint32_t));
      double t0 = now();
      og_bfs(g, arg, hops, parent, &it);
      double t = now() - t0;
      long reach = 0, cs = 0;
      for (uint32_t i = 0; i < N; i++) { reach += hops[i] != 255; cs += (long) hops[i] * parent[i]; }
      dump(out, ".hops.u8", hops, N);
      dump(out, ".parent.u32", parent, N * sizeof(uint32_t));
      printf("{\"app\": \"bfs\", \"exec_s\": %.9f, \"reachable\": %ld, \"checksum\": %ld, \"iters\": %u, "
             "\"nslots\": %u, \"nedges\": %llu}\n", t, reach, cs, it, N, (unsigned long long) og_nedges(g));
      og_free(g);
    }
    else
    {
      og_graph* g = load(path, n, OG_DIRECTED | OG_WEIGHTED);
      uint32_t N = og_nslots(g), it = 0;
      uint32_t* dist = malloc(N * sizeof(uint32_t));
      double t0 = now();
      og_sssp(g, arg, dist, &it);
      double t = now() - t0;
      long reach = 0, cs = 0;
      for (uint32_t i = 0; i < N; i++) { reach += dist[i] != 0x7FFFFFFFu; cs += dist[i]; }
      dump(out, ".dist.u32", dist, N * sizeof(uint32_t));
      printf("{\"app\": \"sssp\", \"exec_s\": %.9f, \"reachable\": %ld, \"checksum\": %ld, \"iters\": %u, "
             "\"nslots\": %u, \"nedges\": %llu}\n", t, reach, cs, it, N, (unsigned long long) og_nedges(g));
      og_free(g);
    }
  }
  else if (!strcmp(app, "cc"))
  {
    const char* out = argv[4];
    og_graph* g = load(path, n, 0);
    uint32_t N = og_nslots(g), it = 0;
    uint32_t* label = malloc(N * sizeof(uint32_t));
    double t0 = now();
    og_cc(g, label, &it);
    double t = now() - t0;
    long cs = 0;
    for (uint32_t i = 0; i < N; i++) cs += label[i];
    dump(out, ".label.u32", label, N * sizeof(uint32_t));
    printf("{\"app\": \"cc\", \"exec_s\": %.9f, \"checksum\": %ld, \"iters\": %u, \"nslots\": %u, "
           "\"nedges\": %llu}\n", t, cs, it, N, (unsigned long long) og_nedges(g));
    og_free(g);
  }
  else if (!strcmp(app, "tc"))
  {
    const char* out = argv[4];
    og_graph* g = load(path, n, OG_DIRECTED | OG_ACYCLIC);
    uint32_t N = og_nslots(g);
    uint32_t* ntri = malloc(N * sizeof(uint32_t));
    uint64_t total = 0;
    double t0 = now();
    og_tc(g, ntri, &total);
    double t = now() - t0;
    dump(out, ".ntri.u32", ntri, N * sizeof(uint32_t));
    printf("{\"app\": \"tc\", \"exec_s\": %.9f, \"triangles\": %llu, \"nslots\": %u, \"nedges\": %llu}\n", t,
           (unsigned long long) total, N, (unsigned long long) og_nedges(g));
    og_free(g);
  }
  else
  {
    fprintf(stderr, "unknown app %s\n", app);
    return 1;
  }
  return 0;
}
