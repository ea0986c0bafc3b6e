// Minimal binary output archive: vectors as (u64 size, raw elements), trivially
// copyable values raw, classes through their serialize() member.  Reference CPU
// build only; both ends of every message are this process, so the layout only
// has to agree with binary_iarchive.hpp.
#ifndef LA3_REFSHIM_BOOST_OARCHIVE
#define LA3_REFSHIM_BOOST_OARCHIVE
#include <cstdint>
#include <ostream>
#include <type_traits>
#include <vector>
namespace boost { namespace archive {
class binary_oarchive
{
  std::ostream& os_;

  template <class T>
  auto save_(const T& v, int) -> decltype(const_cast<T&>(v).serialize(*this, 0u), void())
  { const_cast<T&>(v).serialize(*this, 0u); }

  template <class T>
  void save_(const T& v, long)
  {
    static_assert(std::is_trivially_copyable<T>::value, "refshim: cannot serialize type");
    os_.write(reinterpret_cast<const char*>(&v), sizeof(T));
  }

public:
  explicit binary_oarchive(std::ostream& os) : os_(os) {}

  template <class U, class A>
  void save(const std::vector<U, A>& v)
  {
    uint64_t n = v.size();
    os_.write(reinterpret_cast<const char*>(&n), sizeof(n));
    if (n) os_.write(reinterpret_cast<const char*>(v.data()), (std::streamsize) (n * sizeof(U)));
  }

  template <class A>
  void save(const std::vector<bool, A>& v)  // one byte per element
  {
    uint64_t n = v.size();
    os_.write(reinterpret_cast<const char*>(&n), sizeof(n));
    for (bool b : v) { char c = b ? 1 : 0; os_.write(&c, 1); }
  }

  template <class T>
  void save(const T& v) { save_(v, 0); }

  template <class T>
  binary_oarchive& operator<<(const T& v) { save(v); return *this; }

  template <class T>
  binary_oarchive& operator&(const T& v) { save(v); return *this; }
};
} }
#endif
