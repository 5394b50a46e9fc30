/* Driver for the reference's own 8pac unpack and B-engine header reform
 * (software/aphids/vdif_8pac.c, software/aphids/beng_reform.c), compiled
 * from those sources by oracle/Makefile into oracle/_ref/ref_8pac.
 *
 * TEST INFRASTRUCTURE ONLY: it generates and checks golden vectors for the
 * oracle; the product never runs it.
 *
 * usage: ref_8pac IN OUT N1 [N2 ...]
 *   IN   raw 8pac units (8504 B each), OUT the unpacked, reformed 1056-B
 *   packets; the units are passed in batches of N1, N2, ... units, one
 *   unpack_8pac + beng_reform_headers call per batch, as the ingest thread
 *   does per receive (vdif_in_net_thread.c:291-298).  Prints T0 (as
 *   get_beng_t0 returns it), TPREV and BPREV at the end. */
#include <stdio.h>
#include <stdlib.h>

#include "beng_reform.h"
#include "vdif_8pac.h"

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s IN OUT N1 [N2 ...]\n", argv[0]);
        return 2;
    }
    FILE *fi = fopen(argv[1], "rb");
    FILE *fo = fopen(argv[2], "wb");
    if (!fi || !fo) {
        perror("open");
        return 2;
    }
    for (int a = 3; a < argc; ++a) {
        const long n = strtol(argv[a], NULL, 10);
        if (n <= 0) continue;
        vdif_8pac_packet_t *src = malloc(sizeof(vdif_8pac_packet_t) * (size_t)n);
        vdif_in_packet_t *dst = malloc(sizeof(vdif_in_packet_t) * 8 * (size_t)n);
        if (!src || !dst) return 3;
        if (fread(src, sizeof(vdif_8pac_packet_t), (size_t)n, fi) != (size_t)n) {
            fprintf(stderr, "short input\n");
            return 4;
        }
        unpack_8pac(dst, src, (int)n);
        beng_reform_headers(dst, (int)(8 * n));
        fwrite(dst, sizeof(vdif_in_packet_t), 8 * (size_t)n, fo);
        free(src);
        free(dst);
    }
    fclose(fi);
    fclose(fo);
    beng_timestamp_t t0, tp;
    int64_t bp;
    get_beng_t0(&t0);
    get_beng_tprev(&tp);
    get_beng_bprev(&bp);
    printf("%d %d %d %d %lld %zu\n", t0.sec, t0.clk, tp.sec, tp.clk, (long long)bp, sizeof(vdif_8pac_packet_t));
    return 0;
}
