// Minimal back-insert device (reference CPU build only).
#ifndef LA3_REFSHIM_BOOST_BACK_INSERTER
#define LA3_REFSHIM_BOOST_BACK_INSERTER
namespace boost { namespace iostreams {
template <class Container>
struct back_insert_device
{
  Container* c;
  explicit back_insert_device(Container& c_) : c(&c_) {}
};
} }
#endif
