/* Install-time cache size in elements of the working type (the getf2 cut-off
 * of the recursive LU).  Override with -DREFSHIM_L1C_ELTS=n.  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_CACHE_H
#define REFSHIM_CACHE_H
#ifndef REFSHIM_L1C_ELTS
   #define REFSHIM_L1C_ELTS 4096
#endif
#define L1C_ELTS REFSHIM_L1C_ELTS
#endif
