// Single-rank Boost.MPI communicator stand-in (reference CPU build only).
#ifndef LA3_REFSHIM_BOOST_MPI_COMM
#define LA3_REFSHIM_BOOST_MPI_COMM
namespace boost { namespace mpi { struct communicator {}; } }
#endif
