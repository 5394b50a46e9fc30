/* Driver for the reference's own host-side group assembly and output-header
 * code, compiled from its sources by oracle/Makefile into
 * oracle/_ref/ref_hostlogic:
 *   software/aphids/vdif_in_databuf.c   get_beng_group_index_offset,
 *       insert_vdif_in_beng_group_buffer, check_beng_group_complete,
 *       init_beng_group (:96-167), fill_vdif_header_template (:193-220)
 *   software/aphids/vdif_out_databuf.c  init_vdif_out (:35-64)
 *   software/aphids/beng_reform.c       the T0 timestamp those read
 * The sources are included into this translation unit so that the file-
 * static T0 of beng_reform.c can be set directly.
 *
 * TEST INFRASTRUCTURE ONLY: it generates golden vectors that pin the
 * oracle's restatement; the product never runs it.
 *
 * usage:
 *   ref_hostlogic template SEC CLK NSKIP
 *       T0 = (SEC, CLK); prints "RESULT secs_inre df_num_insec edh_psn" of
 *       fill_vdif_header_template.
 *   ref_hostlogic ingest HDRS OUT N1 [N2 ...]
 *       HDRS: 32-byte packet headers; they arrive in batches of N1, N2, ...
 *       packets and run through the ingest loop of vdif_in_net_thread.c:
 *       340-500 (sort, b_first, per-packet offset / insert / completion,
 *       look-ahead shipping), restated below around the reference's own
 *       per-packet functions.  OUT (int64 little endian): per input packet
 *       its outcome (absolute group number it was inserted into, or -1
 *       invalid, -2 before start, -3 too far ahead, -4 not inserted), then
 *       the shipped groups (absolute number, packets held) in order.
 *   ref_hostlogic outhdr
 *       prints "WORDS w0 .. w7" (hex) of packets 0 and VDIF_OUT_PKTS_PER_BLOCK-1
 *       of channels 0 and 1 after init_vdif_out. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "beng_reform.c"
#include "vdif_in_databuf.c"
#include "vdif_out_databuf.c"

/* the CUDA-side helpers the databuf sources reference; never called here */
int get_bgv_cpu_memory_cuda(beng_group_vdif_buffer_t **b, int i) { (void)b; (void)i; return -1; }
int get_bgv_gpu_memory_cuda(beng_group_vdif_buffer_t **b, int i) { (void)b; (void)i; return -1; }
int transfer_beng_group_to_gpu_cuda(vdif_in_databuf_t *b, int i) { (void)b; (void)i; return -1; }
int check_transfer_beng_group_to_gpu_complete_cuda(vdif_in_databuf_t *b, int i) { (void)b; (void)i; return -1; }
int get_vdg_cpu_memory_cuda(vdif_out_data_group_t **b, int i) { (void)b; (void)i; return -1; }
int transfer_vdif_group_to_cpu_cuda(vdif_out_databuf_t *b, int i) { (void)b; (void)i; return -1; }
int check_transfer_vdif_group_to_cpu_complete_cuda(vdif_out_databuf_t *b, int i) { (void)b; (void)i; return -1; }
hashpipe_databuf_t *hashpipe_databuf_create(int a, int b, size_t c, size_t d, int e) {
    (void)a; (void)b; (void)c; (void)d; (void)e;
    return NULL;
}

#define LOOK_AHEAD 2 /* MAX_INDEX_LOOK_AHEAD, vdif_in_net_thread.c:136 */

typedef struct {
    vdif_in_packet_t pkt;
    int64_t idx;
} rx_t;

/* compar_beng (vdif_in_net_thread.c:48-68): invalid first, then by b; ties
 * by input position so that the run is reproducible */
static int compar_rx(const void *a, const void *b) {
    const rx_t *x = (const rx_t *)a, *y = (const rx_t *)b;
    const int ia = x->pkt.header.w0.invalid, ib = y->pkt.header.w0.invalid;
    if (ia != ib) return ia ? -1 : 1;
    if (!ia) {
        const int64_t ba = get_packet_b_count((vdif_in_header_t *)&x->pkt.header);
        const int64_t bb = get_packet_b_count((vdif_in_header_t *)&y->pkt.header);
        if (ba != bb) return ba < bb ? -1 : 1;
    }
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

static int run_ingest(const char *hdrs, const char *out, int nb, char **batches) {
    FILE *fi = fopen(hdrs, "rb");
    if (!fi) return 2;
    fseek(fi, 0, SEEK_END);
    const int64_t n = ftell(fi) / 32;
    fseek(fi, 0, SEEK_SET);
    int64_t *outcome = malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t *ships = malloc(sizeof(int64_t) * 2 * 4096);
    int n_ships = 0;
    static vdif_in_databuf_t db;
    memset(&db, 0, sizeof(db));
    /* packet stores: sized for the packets a group can receive here */
    beng_group_vdif_buffer_t *store[BENG_GROUPS_IN_BUFFER];
    const size_t store_bytes = sizeof(vdif_in_packet_t) * (size_t)(n < BENG_FRAMES_PER_GROUP * VDIF_PER_BENG_FRAME
                                                                       ? (n > 0 ? n : 1)
                                                                       : BENG_FRAMES_PER_GROUP * VDIF_PER_BENG_FRAME);
    for (int g = 0; g < BENG_GROUPS_IN_BUFFER; ++g) store[g] = malloc(store_bytes);
    int64_t group_no[BENG_GROUPS_IN_BUFFER]; /* absolute group number held by each slot */
    int index_db_out = 0;
    int64_t b_first = -1, next_group = 0, pos = 0;
    for (int a = 0; a < nb; ++a) {
        const int64_t m = strtoll(batches[a], NULL, 10);
        if (m <= 0) continue;
        rx_t *rx = calloc((size_t)m, sizeof(rx_t));
        for (int64_t i = 0; i < m; ++i) {
            if (fread(&rx[i].pkt.header, 32, 1, fi) != 1) return 3;
            rx[i].idx = pos + i;
            outcome[pos + i] = -4;
        }
        pos += m;
        qsort(rx, (size_t)m, sizeof(rx_t), compar_rx);
        int64_t k = 0;
        if (b_first == -1) {
            while (k < m) {
                b_first = get_packet_b_count(&rx[k].pkt.header);
                if (b_first < 0) {
                    outcome[rx[k].idx] = -1;
                    ++k;
                } else {
                    break;
                }
            }
            if (b_first < 0) {
                free(rx);
                continue;
            }
            for (int g = 0; g < BENG_GROUPS_IN_BUFFER; ++g) {
                init_beng_group(db.bgc + g, store[g], store[g], b_first + 1 + BENG_FRAMES_PER_GROUP * g);
                group_no[g] = next_group++;
            }
        }
        while (k < m) {
            vdif_in_packet_t *p = &rx[k].pkt;
            const int off = get_beng_group_index_offset(&db, index_db_out, p);
            int ship = 0;
            if (off < 0) {
                outcome[rx[k].idx] = off == vidErrorPacketInvalid ? -1 : (off == vidErrorPacketBeforeStartTime ? -2 : -3);
                ++k;
                continue;
            }
            if (off > LOOK_AHEAD) {
                ship = 1; /* the oldest group ships incomplete; the packet is examined again */
            } else {
                const int got = insert_vdif_in_beng_group_buffer(&db, index_db_out, off, p);
                if (got > 0) outcome[rx[k].idx] = group_no[(index_db_out + off) % BENG_GROUPS_IN_BUFFER];
                ++k;
                if (check_beng_group_complete(&db, index_db_out)) ship = 1;
            }
            if (ship) {
                const int g = index_db_out;
                ships[2 * n_ships] = group_no[g];
                ships[2 * n_ships + 1] = db.bgc[g].beng_group_vdif_packet_count;
                ++n_ships;
                init_beng_group(db.bgc + g, store[g], store[g],
                                (int64_t)db.bgc[(g + BENG_GROUPS_IN_BUFFER - 1) % BENG_GROUPS_IN_BUFFER]
                                        .bfc[BENG_FRAMES_PER_GROUP - 1]
                                        .b +
                                    1);
                group_no[g] = next_group++;
                index_db_out = (index_db_out + 1) % BENG_GROUPS_IN_BUFFER;
            }
        }
        free(rx);
    }
    fclose(fi);
    FILE *fo = fopen(out, "wb");
    if (!fo) return 2;
    fwrite(&n, sizeof(int64_t), 1, fo);
    fwrite(outcome, sizeof(int64_t), (size_t)n, fo);
    const int64_t ns = n_ships;
    fwrite(&ns, sizeof(int64_t), 1, fo);
    fwrite(ships, sizeof(int64_t), 2 * (size_t)n_ships, fo);
    fclose(fo);
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 5 && strcmp(argv[1], "template") == 0) {
        T0.sec = (int32_t)strtol(argv[2], NULL, 10);
        T0.clk = (int32_t)strtol(argv[3], NULL, 10);
        vdif_in_header_t hdr;
        vdif_in_packet_t pkt;
        memset(&hdr, 0, sizeof(hdr));
        memset(&pkt, 0, sizeof(pkt));
        fill_vdif_header_template(&hdr, &pkt, (int)strtol(argv[4], NULL, 10));
        printf("RESULT %u %u %llu\n", (unsigned)hdr.w0.secs_inre, (unsigned)hdr.w1.df_num_insec,
               (unsigned long long)hdr.edh_psn);
        return 0;
    }
    if (argc >= 5 && strcmp(argv[1], "ingest") == 0) return run_ingest(argv[2], argv[3], argc - 4, argv + 4);
    if (argc >= 2 && strcmp(argv[1], "outhdr") == 0) {
        vdif_out_packet_group_t *vpg[1];
        vpg[0] = malloc(sizeof(vdif_out_packet_group_t));
        if (!vpg[0]) return 3;
        memset(vpg[0], 0xA5, sizeof(vdif_out_packet_group_t));
        init_vdif_out(vpg, 0);
        const int pk[2] = {0, VDIF_OUT_PKTS_PER_BLOCK - 1};
        for (int ch = 0; ch < VDIF_CHAN; ++ch)
            for (int i = 0; i < 2; ++i) {
                const uint32_t *w = (const uint32_t *)&vpg[0]->chan[ch].packets[pk[i]].header;
                printf("WORDS %d %d %08x %08x %08x %08x %08x %08x %08x %08x\n", ch, pk[i], w[0], w[1], w[2], w[3], w[4],
                       w[5], w[6], w[7]);
            }
        free(vpg[0]);
        return 0;
    }
    fprintf(stderr, "usage: %s template SEC CLK NSKIP | ingest HDRS OUT N1 [N2 ...] | outhdr\n", argv[0]);
    return 2;
}
