// Serial stand-in for the MPI datatype traits: the LB headers only name them.
#ifndef HLB_REFSHIM_NET_MPIDATATYPE_H
#define HLB_REFSHIM_NET_MPIDATATYPE_H
typedef int MPI_Datatype;
namespace hemelb::net {
template <class T>
MPI_Datatype MpiDataType() { return 0; }
template <class T>
MPI_Datatype MpiDataType(T const&) { return 0; }
}  // namespace hemelb::net
#endif
