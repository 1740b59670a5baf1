/* Empty stand-in: the extracted Level-3 tester includes it but calls none of
 * the access-major kernels it declares.  TEST INFRASTRUCTURE ONLY. */
#include "atlas_misc.h"
