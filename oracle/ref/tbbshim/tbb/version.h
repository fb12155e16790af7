// Project-written TBB-API shim (test oracle only): version macros.
#ifndef GBLS_TBBSHIM_VERSION_H
#define GBLS_TBBSHIM_VERSION_H
#include "detail/shim_core.h"
#endif
