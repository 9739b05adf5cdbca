/* A stand-in "libXilinxPcgStatic.so" that exports only xJPCG_getErrorString:
 * the loader must report the missing symbols as a dynamic loading error. */
#include "pcg.h"

const char* xJPCG_getErrorString(const XJPCG_Status_t code) { return code == 0 ? "stub success" : "stub error"; }
