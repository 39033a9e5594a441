/*
 * pq_encode.c — RLE / bit-packed hybrid encoder for Parquet dictionary
 * indices (the Parquet format's hybrid encoding), used by the project's
 * Parquet writer to produce test and benchmark files.
 *
 * Layout written: a run of >= 16 equal values becomes an RLE run; everything
 * in between is bit-packed in groups of 8, borrowing up to 7 values from the
 * start of the next RLE run so each bit-packed stretch is a whole number of
 * groups (the final stretch is zero-padded; readers stop at num_values).
 * Bit-packed runs carry at most 63 groups per header.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static int64_t put_varint(uint8_t *out, int64_t pos, uint64_t v) {
    while (v >= 0x80) {
        out[pos++] = (uint8_t)(v | 0x80);
        v >>= 7;
    }
    out[pos++] = (uint8_t)v;
    return pos;
}

/* bit-pack n (multiple of 8) values LSB-first at bit width bw */
static int64_t put_packed(uint8_t *out, int64_t pos, const uint32_t *v, int64_t n, int bw) {
    uint64_t buf = 0;
    int bits = 0;
    for (int64_t i = 0; i < n; i++) {
        buf |= (uint64_t)(bw >= 32 ? v[i] : (v[i] & ((1u << bw) - 1u))) << bits;
        bits += bw;
        while (bits >= 8) {
            out[pos++] = (uint8_t)buf;
            buf >>= 8;
            bits -= 8;
        }
    }
    if (bits > 0) out[pos++] = (uint8_t)buf;
    return pos;
}

static int64_t flush_literals(uint8_t *out, int64_t pos, const uint32_t *lit, int64_t n, int bw) {
    int64_t done = 0;
    while (done < n) {
        int64_t groups = (n - done) / 8;
        if (groups > 63) groups = 63;
        pos = put_varint(out, pos, ((uint64_t)groups << 1) | 1u);
        pos = put_packed(out, pos, lit + done, groups * 8, bw);
        done += groups * 8;
    }
    return pos;
}

/* Encode n indices; returns bytes written (no bit-width byte), or -1 if cap
 * would be exceeded.  scratch must hold n + 8 uint32. */
int64_t pq_rle_encode(const uint32_t *x, int64_t n, int32_t bw, uint8_t *out, int64_t cap, uint32_t *scratch) {
    int64_t pos = 0, nlit = 0, i = 0;
    const int vbytes = (bw + 7) / 8;
    while (i < n) {
        int64_t j = i + 1;
        while (j < n && x[j] == x[i]) j++;
        int64_t L = j - i;
        if (L >= 16) {
            int64_t pad = (8 - (nlit & 7)) & 7;
            for (int64_t k = 0; k < pad; k++) scratch[nlit++] = x[i];
            if (pos + nlit * 4 + 64 > cap) return -1;
            pos = flush_literals(out, pos, scratch, nlit, bw);
            nlit = 0;
            int64_t rl = L - pad;
            pos = put_varint(out, pos, (uint64_t)rl << 1);
            for (int b = 0; b < vbytes; b++) out[pos++] = (uint8_t)(x[i] >> (8 * b));
        } else {
            for (int64_t k = 0; k < L; k++) scratch[nlit++] = x[i];
        }
        i = j;
        if (pos + 64 > cap) return -1;
    }
    if (nlit) {
        int64_t pad = (8 - (nlit & 7)) & 7;
        for (int64_t k = 0; k < pad; k++) scratch[nlit++] = 0;
        if (pos + nlit * 4 + 64 > cap) return -1;
        pos = flush_literals(out, pos, scratch, nlit, bw);
    }
    return pos;
}

/*
 * Snappy raw-block compressor for the writer's SNAPPY column chunks (the
 * published Snappy format: varint uncompressed length, then literal and copy
 * elements).  Greedy: a 4-byte hash of each position finds an earlier match
 * within 65535 bytes; matches become copies of at most 64 bytes (2-byte
 * offsets, or 1-byte offsets for 4..11 bytes within 2047), everything else
 * literals.  Returns the compressed size, or -1 if `cap` is too small
 * (n + n / 6 + 32 always suffices).
 */
static int64_t put_literal(uint8_t *out, int64_t pos, int64_t cap, const uint8_t *p, int64_t len) {
    while (len > 0) {
        const int64_t l = len > 65536 ? 65536 : len;
        const uint32_t m = (uint32_t)(l - 1);
        if (pos + 3 + l > cap) return -1;
        if (m < 60) {
            out[pos++] = (uint8_t)(m << 2);
        } else if (m < 256) {
            out[pos++] = (uint8_t)(60 << 2);
            out[pos++] = (uint8_t)m;
        } else {
            out[pos++] = (uint8_t)(61 << 2);
            out[pos++] = (uint8_t)m;
            out[pos++] = (uint8_t)(m >> 8);
        }
        memcpy(out + pos, p, (size_t)l);
        pos += l;
        p += l;
        len -= l;
    }
    return pos;
}

static inline uint32_t load32(const uint8_t *p) {
    uint32_t v;
    memcpy(&v, p, 4);
    return v;
}

int64_t pq_snappy_compress(const uint8_t *src, int64_t n, uint8_t *out, int64_t cap, int32_t *table) {
    enum { HB = 14 };
    int64_t pos = 0;
    if (cap < 10) return -1;
    pos = put_varint(out, pos, (uint64_t)n);
    for (int i = 0; i < (1 << HB); i++) table[i] = -1;
    int64_t i = 0, lit = 0;
    while (i + 4 <= n) {
        const uint32_t w = load32(src + i);
        const uint32_t h = (w * 0x1e35a7bdu) >> (32 - HB);
        const int64_t cand = table[h];
        table[h] = (int32_t)i;
        if (cand >= 0 && i - cand <= 65535 && load32(src + cand) == w) {
            int64_t len = 4;
            while (len < 64 && i + len < n && src[cand + len] == src[i + len]) len++;
            if ((pos = put_literal(out, pos, cap, src + lit, i - lit)) < 0) return -1;
            const int64_t off = i - cand;
            if (pos + 3 > cap) return -1;
            if (len <= 11 && off < 2048) {
                out[pos++] = (uint8_t)(1 | ((len - 4) << 2) | ((off >> 8) << 5));
                out[pos++] = (uint8_t)off;
            } else {
                out[pos++] = (uint8_t)(2 | ((len - 1) << 2));
                out[pos++] = (uint8_t)off;
                out[pos++] = (uint8_t)(off >> 8);
            }
            i += len;
            lit = i;
        } else {
            i++;
        }
    }
    if ((pos = put_literal(out, pos, cap, src + lit, n - lit)) < 0) return -1;
    return pos;
}

/*
 * ZSTD frame compressor for the writer's ZSTD column chunks (the published
 * format, RFC 8878): one frame (single segment, 4-byte content size, no
 * checksum) of blocks of at most 128 KB.  Each block is matched greedily (a
 * 4-byte hash of each position finds an earlier match anywhere in the frame)
 * and written as a compressed block with raw literals and its sequences
 * coded with the format's predefined FSE tables, or as a raw block when that
 * is not smaller.  Returns the compressed size, or -1 if `cap` is too small
 * (n + n / 128 + 64 always suffices).
 */
typedef struct {
    uint8_t *out;
    int64_t cap, pos;
    uint64_t acc;
    int nacc, bad;
} ZBitW;

static void zbw_add(ZBitW *w, uint64_t v, int nb) {
    if (nb == 0) return;
    w->acc |= (v & ((nb >= 64) ? ~0ull : ((1ull << nb) - 1))) << w->nacc;
    w->nacc += nb;
    while (w->nacc >= 8) {
        if (w->pos >= w->cap) {
            w->bad = 1;
            return;
        }
        w->out[w->pos++] = (uint8_t)w->acc;
        w->acc >>= 8;
        w->nacc -= 8;
    }
}

static void zbw_close(ZBitW *w) {  /* the end marker bit, then the last partial byte */
    zbw_add(w, 1, 1);
    if (w->nacc > 0) {
        if (w->pos >= w->cap) {
            w->bad = 1;
            return;
        }
        w->out[w->pos++] = (uint8_t)w->acc;
        w->acc = 0;
        w->nacc = 0;
    }
}

static int zhighbit(uint32_t v) {
    int r = 0;
    while (v >>= 1) r++;
    return r;
}

/* FSE encoding table of one predefined distribution */
typedef struct {
    uint16_t next[64];  /* state values [size, 2 size) sorted by symbol */
    int32_t dnb[64], dfs[64];
    int log;
} ZEnc;

static void zenc_build(ZEnc *E, const int16_t *norm, int nsym, int log) {
    const int size = 1 << log, mask = size - 1;
    int high = size - 1, cumul[65], pos = 0, total = 0;
    uint8_t sym[64];
    E->log = log;
    cumul[0] = 0;
    for (int s = 0; s < nsym; s++) {
        if (norm[s] == -1) {
            cumul[s + 1] = cumul[s] + 1;
            sym[high--] = (uint8_t)s;
        } else {
            cumul[s + 1] = cumul[s] + norm[s];
        }
    }
    const int step = (size >> 1) + (size >> 3) + 3;
    for (int s = 0; s < nsym; s++)
        for (int k = 0; k < norm[s]; k++) {
            sym[pos] = (uint8_t)s;
            do {
                pos = (pos + step) & mask;
            } while (pos > high);
        }
    for (int u = 0; u < size; u++) E->next[cumul[sym[u]]++] = (uint16_t)(size + u);
    for (int s = 0; s < nsym; s++) {
        const int n = norm[s];
        if (n == 0) {
            E->dnb[s] = ((log + 1) << 16) - size;
            E->dfs[s] = 0;
        } else if (n == -1 || n == 1) {
            E->dnb[s] = (log << 16) - size;
            E->dfs[s] = total - 1;
            total++;
        } else {
            const int mbo = log - zhighbit((uint32_t)n - 1);
            E->dnb[s] = (mbo << 16) - (n << mbo);
            E->dfs[s] = total - n;
            total += n;
        }
    }
}

static uint32_t zenc_init(const ZEnc *E, int s) {
    const int nb = (E->dnb[s] + (1 << 15)) >> 16;
    const uint32_t v = (uint32_t)((nb << 16) - E->dnb[s]);
    return E->next[(v >> nb) + E->dfs[s]];
}

static uint32_t zenc_sym(const ZEnc *E, ZBitW *w, uint32_t state, int s) {
    const int nb = (int)((state + (uint32_t)E->dnb[s]) >> 16);
    zbw_add(w, state, nb);
    return E->next[(state >> nb) + E->dfs[s]];
}

static const int16_t ZLL_NORM[36] = {4, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 1, 1, 1, 2, 2,
                                     2, 2, 2, 2, 2, 2, 2, 3, 2, 1, 1, 1, 1, 1, -1, -1, -1, -1};
static const int16_t ZML_NORM[53] = {1, 4, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1};
static const int16_t ZOF_NORM[29] = {1, 1, 1, 1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                     1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1};
static const uint32_t ZLL_BASE[36] = {0,  1,  2,  3,  4,  5,   6,   7,   8,    9,    10,   11,   12,
                                      13, 14, 15, 16, 18, 20,  22,  24,  28,   32,   40,   48,   64,
                                      128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 65536};
static const uint8_t ZLL_BITS[36] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,  0,  1,  1,
                                     1, 1, 2, 2, 3, 3, 4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16};
static const uint32_t ZML_BASE[53] = {3,  4,  5,  6,  7,  8,  9,  10, 11, 12, 13,  14,  15,   16,   17,   18,   19,   20,
                                      21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31,  32,  33,   34,   35,   37,   39,   41,
                                      43, 47, 51, 59, 67, 83, 99, 131, 259, 515, 1027, 2051, 4099, 8195, 16387, 32771, 65539};
static const uint8_t ZML_BITS[53] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                     0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3, 4, 4, 5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16};

static int zcode(const uint32_t *base, int ncodes, uint32_t v) {  /* the largest code whose baseline <= v */
    int c = ncodes - 1;
    while (c > 0 && base[c] > v) c--;
    return c;
}

typedef struct {
    uint32_t ll, ml, off;
} ZSeq;

/* One block [b0, b1) of src as a compressed block body at out; its size or -1 (does not fit). */
static int64_t zblock(const uint8_t *src, int64_t b0, int64_t b1, int32_t *table, ZSeq *seqs, uint8_t *out, int64_t cap,
                      const ZEnc *ell, const ZEnc *eml, const ZEnc *eof) {
    enum { HB = 16 };
    int64_t i = b0, lit = b0, nseq = 0, nlit = 0;
    /* literals are gathered at the end of out, then moved */
    uint8_t *lits = out + cap - (b1 - b0);
    if (cap < (b1 - b0) + 16) return -1;
    while (i + 4 <= b1) {
        const uint32_t w = load32(src + i);
        const uint32_t h = (w * 0x9E3779B1u) >> (32 - HB);
        const int64_t cand = table[h];
        table[h] = (int32_t)i;
        if (cand >= 0 && i - cand < (1 << 27) && load32(src + cand) == w) {
            int64_t len = 4;
            while (i + len < b1 && src[cand + len] == src[i + len]) len++;
            memcpy(lits + nlit, src + lit, (size_t)(i - lit));
            nlit += i - lit;
            seqs[nseq].ll = (uint32_t)(i - lit);
            seqs[nseq].ml = (uint32_t)len;
            seqs[nseq].off = (uint32_t)(i - cand);
            nseq++;
            i += len;
            lit = i;
        } else {
            i++;
        }
    }
    memcpy(lits + nlit, src + lit, (size_t)(b1 - lit));
    nlit += b1 - lit;
    /* literals section: raw */
    int64_t pos = 0;
    if (nlit < 32) {
        out[pos++] = (uint8_t)(nlit << 3);
    } else if (nlit < 4096) {
        out[pos++] = (uint8_t)(((nlit & 15) << 4) | (1 << 2));
        out[pos++] = (uint8_t)(nlit >> 4);
    } else {
        out[pos++] = (uint8_t)(((nlit & 15) << 4) | (3 << 2));
        out[pos++] = (uint8_t)(nlit >> 4);
        out[pos++] = (uint8_t)(nlit >> 12);
    }
    if (pos + nlit + 8 > cap - (b1 - b0)) return -1;  /* must not reach the gathered literals' end */
    memmove(out + pos, lits, (size_t)nlit);
    pos += nlit;
    /* sequences section */
    if (nseq < 128) {
        out[pos++] = (uint8_t)nseq;
    } else if (nseq < 0x7F00) {
        out[pos++] = (uint8_t)((nseq >> 8) + 128);
        out[pos++] = (uint8_t)nseq;
    } else {
        out[pos++] = 255;
        out[pos++] = (uint8_t)(nseq - 0x7F00);
        out[pos++] = (uint8_t)((nseq - 0x7F00) >> 8);
    }
    if (nseq == 0) return pos;
    out[pos++] = 0;  /* literal lengths, offsets, match lengths: predefined tables */
    ZBitW bw = {out, cap, pos, 0, 0, 0};
    uint32_t sll = 0, sml = 0, sof = 0;
    for (int64_t q = nseq - 1; q >= 0; q--) {
        const ZSeq *z = &seqs[q];
        const int llc = zcode(ZLL_BASE, 36, z->ll), mlc = zcode(ZML_BASE, 53, z->ml);
        const uint32_t ofv = z->off + 3;
        const int ofc = zhighbit(ofv);
        if (q == nseq - 1) {
            sml = zenc_init(eml, mlc);
            sof = zenc_init(eof, ofc);
            sll = zenc_init(ell, llc);
        } else {
            sof = zenc_sym(eof, &bw, sof, ofc);
            sml = zenc_sym(eml, &bw, sml, mlc);
            sll = zenc_sym(ell, &bw, sll, llc);
        }
        zbw_add(&bw, z->ll - ZLL_BASE[llc], ZLL_BITS[llc]);
        zbw_add(&bw, z->ml - ZML_BASE[mlc], ZML_BITS[mlc]);
        zbw_add(&bw, ofv - (1u << ofc), ofc);
    }
    zbw_add(&bw, sml, eml->log);
    zbw_add(&bw, sof, eof->log);
    zbw_add(&bw, sll, ell->log);
    zbw_close(&bw);
    return bw.bad ? -1 : bw.pos;
}

int64_t pq_zstd_compress(const uint8_t *src, int64_t n, uint8_t *out, int64_t cap, int32_t *table) {
    enum { HB = 16, BLOCK = 131072 };
    static ZEnc ell, eml, eof;
    static int built = 0;
    if (!built) {
        zenc_build(&ell, ZLL_NORM, 36, 6);
        zenc_build(&eml, ZML_NORM, 53, 6);
        zenc_build(&eof, ZOF_NORM, 29, 5);
        built = 1;
    }
    if (cap < 16) return -1;
    int64_t pos = 0;
    out[pos++] = 0x28;
    out[pos++] = 0xB5;
    out[pos++] = 0x2F;
    out[pos++] = 0xFD;
    out[pos++] = 0xA0;  /* 4-byte content size, single segment */
    for (int k = 0; k < 4; k++) out[pos++] = (uint8_t)((uint64_t)n >> (8 * k));
    for (int i = 0; i < (1 << HB); i++) table[i] = -1;
    ZSeq *seqs = (ZSeq *)malloc(sizeof(ZSeq) * (BLOCK / 4 + 8));
    uint8_t *tmp = (uint8_t *)malloc((size_t)BLOCK * 2 + 64);
    if (!seqs || !tmp) {
        free(seqs);
        free(tmp);
        return -1;
    }
    int64_t b0 = 0;
    do {
        const int64_t b1 = n - b0 > BLOCK ? b0 + BLOCK : n;
        const int last = b1 == n;
        const int64_t csz = b1 > b0 ? zblock(src, b0, b1, table, seqs, tmp, (int64_t)BLOCK * 2 + 64, &ell, &eml, &eof)
                                     : -1;
        const int raw = csz < 0 || csz >= b1 - b0;
        const int64_t bsz = raw ? b1 - b0 : csz;
        if (pos + 3 + bsz > cap) {
            free(seqs);
            free(tmp);
            return -1;
        }
        const uint32_t bh = (uint32_t)last | ((raw ? 0u : 2u) << 1) | ((uint32_t)bsz << 3);
        out[pos++] = (uint8_t)bh;
        out[pos++] = (uint8_t)(bh >> 8);
        out[pos++] = (uint8_t)(bh >> 16);
        memcpy(out + pos, raw ? src + b0 : tmp, (size_t)bsz);
        pos += bsz;
        b0 = b1;
    } while (b0 < n);
    free(seqs);
    free(tmp);
    return pos;
}
