/* Host stand-in for "device_launch_parameters.h" (see ref_stub.h). */
#ifndef BDREF_DLP_STUB_H
#define BDREF_DLP_STUB_H
#include "../ref_stub.h"
#endif
