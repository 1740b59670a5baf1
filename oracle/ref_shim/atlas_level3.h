/* Empty stand-in: the extracted routines reach Level 1-3 through refshim_cblas.h.
 * TEST INFRASTRUCTURE ONLY. */
#include "atlas_misc.h"
