// Minimal iostreams: an ostream appending to a string, an istream over a char
// array (reference CPU build only).
#ifndef LA3_REFSHIM_BOOST_STREAM
#define LA3_REFSHIM_BOOST_STREAM
#include <cstddef>
#include <istream>
#include <ostream>
#include <streambuf>
#include <string>
#include "boost/iostreams/device/back_inserter.hpp"
namespace boost { namespace iostreams {
template <class Ch>
struct basic_array_source
{
  const Ch* p;
  std::size_t n;
  basic_array_source(const Ch* p_, std::size_t n_) : p(p_), n(n_) {}
};

template <class Device>
class stream;

class la3_append_buf : public std::streambuf
{
  std::string* s_;
protected:
  int_type overflow(int_type ch) override
  {
    if (ch != traits_type::eof()) s_->push_back((char) ch);
    return ch;
  }
  std::streamsize xsputn(const char* p, std::streamsize n) override
  {
    s_->append(p, (std::size_t) n);
    return n;
  }
public:
  explicit la3_append_buf(std::string* s) : s_(s) {}
};

class la3_array_buf : public std::streambuf
{
public:
  la3_array_buf(const char* p, std::size_t n)
  {
    char* b = const_cast<char*>(p);
    setg(b, b, b + n);
  }
};

template <>
class stream<back_insert_device<std::string>> : public std::ostream
{
  la3_append_buf buf_;
public:
  explicit stream(back_insert_device<std::string>& d) : std::ostream(nullptr), buf_(d.c)
  { rdbuf(&buf_); }
};

template <>
class stream<basic_array_source<char>> : public std::istream
{
  la3_array_buf buf_;
public:
  explicit stream(basic_array_source<char>& d) : std::istream(nullptr), buf_(d.p, d.n)
  { rdbuf(&buf_); }
};
} }
#endif
