/* Stand-in for the tuned build's dipgen_view.h: the blocking constants
 * the extracted getri routines name.  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_DIPGEN_VIEW_H
#define REFSHIM_DIPGEN_VIEW_H
#define ATL_VWipgen_100LCMMN 4
#define ATL_VWipgen_98KB 64
#endif
