// Minimal stand-in for Boost.Serialization's access class (reference CPU build only).
#ifndef LA3_REFSHIM_BOOST_SER_ACCESS
#define LA3_REFSHIM_BOOST_SER_ACCESS
namespace boost { namespace serialization { class access {}; } }
#endif
