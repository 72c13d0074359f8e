// Empty: the iolet sources include it but the LB update does not use it.
#ifndef HLB_REFSHIM_NET_IOCOMMUNICATOR_H
#define HLB_REFSHIM_NET_IOCOMMUNICATOR_H
#endif
