/* Minimal stand-in (see mlvalues.h): bem3d_stubs.c includes this header but
 * uses nothing from it. */
#include "mlvalues.h"
