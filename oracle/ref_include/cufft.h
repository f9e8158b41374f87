/* Host stand-in for <cufft.h>: only the complex type the reference's kernels
 * use (W:268-302).  The transform itself is done by the harness. */
#ifndef BDREF_CUFFT_STUB_H
#define BDREF_CUFFT_STUB_H
#include "../ref_stub.h"
#endif
