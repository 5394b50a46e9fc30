/* Empty stand-in for the hashpipe library header, which the reference's
 * databuf sources include; the functions the oracle drivers call use none
 * of it.  TEST INFRASTRUCTURE ONLY. */
#ifndef SDBE_STUB_HASHPIPE_H
#define SDBE_STUB_HASHPIPE_H
#endif
