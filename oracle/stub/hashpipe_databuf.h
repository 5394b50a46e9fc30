/* Minimal stand-in for the hashpipe databuf header: the type and the one
 * declaration the reference's databuf sources name.  The oracle drivers
 * never call it.  TEST INFRASTRUCTURE ONLY. */
#ifndef SDBE_STUB_HASHPIPE_DATABUF_H
#define SDBE_STUB_HASHPIPE_DATABUF_H
#include <stddef.h>
typedef struct hashpipe_databuf {
    char opaque[64];
} hashpipe_databuf_t;
hashpipe_databuf_t *hashpipe_databuf_create(int instance_id, int databuf_id, size_t header_size, size_t block_size,
                                            int n_block);
#endif
