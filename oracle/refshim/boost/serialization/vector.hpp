// std::vector support lives in the archive stand-ins (reference CPU build only).
#ifndef LA3_REFSHIM_BOOST_SER_VECTOR
#define LA3_REFSHIM_BOOST_SER_VECTOR
#include <vector>
#endif
