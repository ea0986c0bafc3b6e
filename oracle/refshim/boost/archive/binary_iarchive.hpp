// Minimal binary input archive matching binary_oarchive.hpp (reference CPU build only).
#ifndef LA3_REFSHIM_BOOST_IARCHIVE
#define LA3_REFSHIM_BOOST_IARCHIVE
#include <cstdint>
#include <istream>
#include <type_traits>
#include <vector>
namespace boost { namespace archive {
class binary_iarchive
{
  std::istream& is_;

  template <class T>
  auto load_(T& v, int) -> decltype(v.serialize(*this, 0u), void())
  { v.serialize(*this, 0u); }

  template <class T>
  void load_(T& v, long)
  {
    static_assert(std::is_trivially_copyable<T>::value, "refshim: cannot deserialize type");
    is_.read(reinterpret_cast<char*>(&v), sizeof(T));
  }

public:
  explicit binary_iarchive(std::istream& is) : is_(is) {}

  template <class U, class A>
  void load(std::vector<U, A>& v)
  {
    uint64_t n = 0;
    is_.read(reinterpret_cast<char*>(&n), sizeof(n));
    v.resize(n);
    if (n) is_.read(reinterpret_cast<char*>(v.data()), (std::streamsize) (n * sizeof(U)));
  }

  template <class A>
  void load(std::vector<bool, A>& v)  // one byte per element
  {
    uint64_t n = 0;
    is_.read(reinterpret_cast<char*>(&n), sizeof(n));
    v.resize(n);
    for (uint64_t i = 0; i < n; i++) { char c = 0; is_.read(&c, 1); v[i] = c != 0; }
  }

  template <class T>
  void load(T& v) { load_(v, 0); }

  template <class T>
  binary_iarchive& operator>>(T& v) { load(v); return *this; }

  template <class T>
  binary_iarchive& operator&(T& v) { load(v); return *this; }
};
} }
#endif
