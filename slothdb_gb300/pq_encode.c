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
