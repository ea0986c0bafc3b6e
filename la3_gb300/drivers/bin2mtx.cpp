// bin2mtx <filepath_in> <filepath_out> [-hi[o]] [-wi] [-wo[r]]
// LA3 binary records (optional 16-byte header) to Matrix Market text lines
// "i j [w]" (tools/bin2mtx.cpp:11-96): -wi reads a uint32 weight per record,
// -wo writes one (1 when not read; -wor writes 1 + rand() % 128 after
// srand(0), the reference tool's sequence); -hio writes the "n m nnz" line.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>

int main(int argc, char** argv)
{
  std::cout << "Convert graph from binary (with optional header: uint:n uint:m ulong:nnz) pairs (uint:i uint:j) or "
               "triples (uint:i uint:j uint:w) to Matrix Market (with optional header: n m nnz) pairs (i j) or "
               "triples (i j w). \n";
  std::cout << "Usage: " << argv[0] << " <filepath_in> <filepath_out> \n"
            << "\t [-hi[o]]  read in header [and write [o]ut]\n"
            << "\t [-wi]     read in edge weights (must be int)\n"
            << "\t [-wo[r]]  write out edge weights (int) \n"
            << "\t           (by default 1, or rand [1,128] if [r]).\n";
  if (argc < 3) return 1;
  bool header_in = false, header_out = false, weights_in = false, weights_out = false, weights_rand = false;
  for (int a = 3; a < argc; a++)
  {
    const std::string o = argv[a];
    if (o == "-hi" || o == "-hio") header_in = true;
    if (o == "-hio") header_out = true;
    if (o == "-wi") weights_in = true;
    if (o == "-wo" || o == "-wor") weights_out = true;
    if (o == "-wor") weights_rand = true;
  }
  std::ifstream in(argv[1], std::ios::binary);
  if (!in)
  {
    std::fprintf(stderr, "cannot open %s\n", argv[1]);
    return 1;
  }
  std::ofstream out(argv[2]);
  if (header_in)
  {
    uint32_t n = 0, m = 0;
    uint64_t nnz = 0;
    in.read((char*) &n, 4);
    in.read((char*) &m, 4);
    in.read((char*) &nnz, 8);
    std::cout << "Header: " << n << " " << m << " " << nnz << "\n";
    if (header_out) out << n << " " << m << " " << nnz << "\n";
  }
  std::srand(0);
  uint32_t i = 0, j = 0, wi = 1;
  while (in.read((char*) &i, 4) && in.read((char*) &j, 4))
  {
    out << i << " " << j;
    if (weights_in) in.read((char*) &wi, 4);
    if (weights_out)
    {
      if (weights_rand) wi = 1u + (uint32_t) (std::rand() % 128);
      out << " " << wi;
    }
    out << "\n";
  }
  return 0;
}
