// mtx2bin <filepath_in> <filepath_out> [-hi[o]] [-wi] [-wo{i|d}]
// Matrix Market text (optional "n m nnz" header line, then "i j [w]" lines;
// lines starting with % or # before the data are comments) to LA3 binary
// records (tools/mtx2bin.cpp:11-116): uint32 pairs, or triples with a uint32
// (-woi) or double (-wod) weight; the 16-byte header with -hio.  Weights that
// are written but not read are 1 + rand() % 128 after srand(0), the same
// sequence the reference tool writes.  The header is read from the first
// non-comment line.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

int main(int argc, char** argv)
{
  std::cout << "Convert graph from Matrix Market (with optional header: n m nnz) pairs (i j) or triples (i j w) "
               "to binary (with optional header: uint:n uint:m ulong:nnz) pairs (uint:i uint:j) or triples "
               "(uint:i uint:j uint:w). \n";
  std::cout << "Usage: " << argv[0] << " <filepath_in> <filepath_out> \n"
            << "\t [-hi[o]]    read in first non-comment line as header [and write [o]ut]\n"
            << "\t [-wi]       read in edge weights (must be int or double) \n"
            << "\t [-wo{i|d}]  write out edge weights ({i}nt/{d}ouble) \n"
            << "\t             (rand [1,128] if none given)\n";
  if (argc < 3) return 1;
  bool header_in = false, header_out = false, weights_in = false, weights_out = false, weights_int = false;
  for (int a = 3; a < argc; a++)
  {
    const std::string o = argv[a];
    if (o == "-hi" || o == "-hio") header_in = true;
    if (o == "-hio") header_out = true;
    if (o == "-wi") weights_in = true;
    if (o == "-woi" || o == "-wod") weights_out = true;
    if (o == "-woi") weights_int = true;
  }
  const bool weights_rand = !weights_in && weights_out;
  std::ifstream in(argv[1]);
  if (!in)
  {
    std::fprintf(stderr, "cannot open %s\n", argv[1]);
    return 1;
  }
  std::ofstream out(argv[2], std::ios::binary);
  while (in.peek() == '%' || in.peek() == '#')
  {
    std::string skip;
    std::getline(in, skip);
  }
  if (header_in)
  {
    uint32_t n = 0, m = 0;
    uint64_t nnz = 0;
    in >> n >> m >> nnz;
    std::cout << "Header: " << n << " " << m << " " << nnz << "\n";
    if (header_out)
    {
      out.write((const char*) &n, 4);
      out.write((const char*) &m, 4);
      out.write((const char*) &nnz, 8);
    }
  }
  std::srand(0);
  uint32_t i = 0, j = 0;
  double wd = 1;
  while (in >> i >> j)
  {
    out.write((const char*) &i, 4);
    out.write((const char*) &j, 4);
    if (weights_in) in >> wd;
    if (weights_out)
    {
      if (weights_rand) wd = 1 + (std::rand() % 128);
      if (weights_int)
      {
        const uint32_t wi = (uint32_t) wd;
        out.write((const char*) &wi, 4);
      }
      else
        out.write((const char*) &wd, 8);
    }
  }
  return 0;
}
