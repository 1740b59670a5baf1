/* The stand-in configuration header of the reference build, plus the Level-1
 * prototypes the tester programs expect it to bring in.
 * TEST INFRASTRUCTURE ONLY. */
#include "../atlas_misc.h"
#include "atlas_level1.h"
