// Stand-in for GundamUtils.h: the two macros the likelihood classes use, and
// the logger GUNDAM's own header brings in.
#ifndef GW_REF_STUB_GUNDAM_UTILS_H
#define GW_REF_STUB_GUNDAM_UTILS_H
#include "Logger.h"
#define GUNDAM_UNLIKELY_COMPILER_FLAG
#define HAS_CPP_17 1
#endif
