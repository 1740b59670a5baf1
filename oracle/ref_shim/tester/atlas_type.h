/* Size of a C long, which the reference's bit-vector header picks its word
 * size from (an install-time constant in the reference).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_TYPE_H
#define REFSHIM_TYPE_H
#define ATL_LSIZE __SIZEOF_LONG__
#endif
