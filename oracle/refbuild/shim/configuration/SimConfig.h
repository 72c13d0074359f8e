// Empty: the iolet sources include it but the LB update does not use it.
#ifndef HLB_REFSHIM_CONFIGURATION_SIMCONFIG_H
#define HLB_REFSHIM_CONFIGURATION_SIMCONFIG_H
#endif
