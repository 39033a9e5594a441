// gb_zstd.h — a ZSTD frame decoder for Parquet's ZSTD pages (codec 6), the
// ZstdDecompress side of src/storage/parquet.cpp:693-736 (which calls the
// vendored zstd library).  Written from the published format, RFC 8878:
// frames of Raw / RLE / Compressed blocks; a compressed block holds a
// literals section (raw, RLE, or Huffman-coded in one or four streams,
// possibly reusing the previous block's table) and a sequences section
// (literal length, match length and offset codes decoded with three FSE
// state machines from one backward bit stream, tables predefined, RLE,
// described in the block, or repeated; three repeat offsets).
//
// Header-only and __host__ __device__: the page inflate runs it on one lane
// per page; the same code built for the host is what the CPU tests check
// against another implementation.  Every read and write is bounds-checked
// against the source, the destination and the scratch: a malformed frame
// returns -1, never a read or write outside them.
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __CUDACC__
#define ZS_HD __host__ __device__ __forceinline__
// Table builders run once per block: kept out of line on the device so
// that their registers do not add to the sequence loop's
#define ZS_COLD __host__ __device__ __noinline__
#else
#define ZS_HD inline
#define ZS_COLD inline
#endif

namespace gbz {

enum : uint32_t {
    ZS_HUF_LOG = 11,      // longest Huffman code of a literals table
    ZS_LL_LOG = 9,        // largest table accuracy of literal lengths
    ZS_ML_LOG = 9,        // ... of match lengths
    ZS_OF_LOG = 8,        // ... of offset codes
    ZS_BLOCK_MAX = 131072,
};

// Scratch of one decode (13.3 KB): the Huffman table, the three sequence
// tables with the lengths' baselines per cell, and the Huffman weights'
// table.  A block's Huffman or RLE literals are decoded into the end of the
// destination, dst[cap - literals, cap) (raw literals are read where they
// lie in the frame): the sequences write at or below the next literal they
// read (their output before the block's end is at most cap - literals + the
// literals read so far), so the literals are consumed before they are
// overwritten.
struct ZsScratch {
    uint16_t huf[1u << ZS_HUF_LOG];  // (symbol << 8) | code length
    uint32_t ll[1u << ZS_LL_LOG], ml[1u << ZS_ML_LOG], of[1u << ZS_OF_LOG];
    // per cell of ll / ml: the length's baseline | its extra bits << 24
    uint32_t llx[1u << ZS_LL_LOG], mlx[1u << ZS_ML_LOG];
    uint32_t wt[64];                 // the Huffman weights' FSE table (accuracy <= 6)
};

// A table cell: symbol (8 bits) | bits to read (8) | baseline of the next state (16).
ZS_HD uint32_t zs_cell(uint32_t sym, uint32_t nb, uint32_t base) { return sym | (nb << 8) | (base << 16); }

ZS_HD int zs_highbit(uint32_t v) {  // index of the highest set bit, v > 0
    int r = 0;
    while (v >>= 1) r++;
    return r;
}

// Bits [pos, pos + n) of the little-endian bit string src[0, size), n <= 32;
// bits outside it read as 0.
ZS_HD uint32_t zs_bits(const uint8_t *src, int64_t size, int64_t pos, int n) {
    if (n == 0) return 0;
    uint64_t v = 0;
    const int64_t b0 = pos >= 0 ? pos >> 3 : -((-pos + 7) >> 3);
    for (int k = 0; k < 6; k++) {  // bytes b0 .. b0 + 5 cover any 32 bits
        const int64_t b = b0 + k;
        if (b >= 0 && b < size) v |= (uint64_t)src[b] << (8 * k);
    }
    const int sh = (int)(pos - b0 * 8);
    return (uint32_t)((v >> sh) & ((n >= 32) ? 0xffffffffull : ((1ull << n) - 1)));
}

// A backward bit stream (FSE and Huffman streams): read from its end, below
// the highest set bit of its last byte.  The 64 bits [wlo, wlo + 64) are
// kept in `win` (bits outside the stream as 0) and reloaded, 8 bytes at a
// time, when a read leaves them.
struct ZsBack {
    const uint8_t *src;
    int32_t size;  // bytes (a stream lies inside one block: at most 128 KB)
    int32_t pos;   // bits not yet read; < 0 once more were read than the stream holds
    int32_t wlo;   // first bit of the window (a multiple of 8)
    uint64_t win;
};

ZS_HD void zs_back_load(ZsBack &b, int32_t top) {  // a window that holds the bits below `top`
    int32_t lo = top - 64;  // rounded up to a byte: the window still reaches `top`
    lo = lo >= 0 ? ((lo + 7) >> 3) << 3 : -((-lo) >> 3) * 8;
    b.wlo = lo;
    uint64_t v = 0;
    const int32_t b0 = lo >> 3;  // exact: lo is a multiple of 8
    if (b0 >= 0 && b0 + 8 <= b.size) {
        for (int k = 0; k < 8; k++) v |= (uint64_t)b.src[b0 + k] << (8 * k);
    } else {
        for (int k = 0; k < 8; k++) {
            const int32_t i = b0 + k;
            if (i >= 0 && i < b.size) v |= (uint64_t)b.src[i] << (8 * k);
        }
    }
    b.win = v;
}

ZS_HD bool zs_back_init(ZsBack &b, const uint8_t *src, int64_t size) {
    if (size <= 0 || size > (int64_t)ZS_BLOCK_MAX || src[size - 1] == 0) return false;
    b.src = src;
    b.size = (int32_t)size;
    b.pos = (b.size - 1) * 8 + zs_highbit(src[size - 1]);
    zs_back_load(b, b.pos);
    return true;
}

// Bits [p, p + n) of the stream, n <= 32.
ZS_HD uint32_t zs_back_bits(ZsBack &b, int32_t p, int n) {
    if (n == 0) return 0;
    if (p < b.wlo || p + n > b.wlo + 64) zs_back_load(b, p + n);
    return (uint32_t)((b.win >> (p - b.wlo)) & ((1ull << n) - 1));
}

ZS_HD uint32_t zs_read(ZsBack &b, int n) {
    b.pos -= n;
    return zs_back_bits(b, b.pos, n);
}

ZS_HD uint32_t zs_peek(ZsBack &b, int n) { return zs_back_bits(b, b.pos - n, n); }

// FSE decoding table of `log` accuracy from normalized counts (-1: "less
// than one", a cell of its own at the top of the table).
ZS_HD bool zs_fse_build(uint32_t *tab, int log, const int16_t *norm, int nsym) {
    const uint32_t size = 1u << log, mask = size - 1;
    uint16_t next[256];
    int32_t high = (int32_t)size - 1;
    for (int s = 0; s < nsym; s++) {
        if (norm[s] == -1) {
            if (high < 0) return false;
            tab[high--] = (uint32_t)s;
            next[s] = 1;
        } else {
            next[s] = (uint16_t)norm[s];
        }
    }
    uint32_t pos = 0;
    const uint32_t step = (size >> 1) + (size >> 3) + 3;
    for (int s = 0; s < nsym; s++) {
        for (int k = 0; k < norm[s]; k++) {
            if (high < 0) return false;
            tab[pos] = (uint32_t)s;
            do {
                pos = (pos + step) & mask;
            } while ((int32_t)pos > high);
        }
    }
    if (pos != 0) return false;  // the counts did not fill the table
    // every cell: the next state's baseline and bits (a "less than one"
    // symbol's single cell reads all `log` bits from baseline 0)
    for (uint32_t i = 0; i < size; i++) {
        const uint32_t s = tab[i] & 0xffu;
        const uint32_t x = next[s]++;
        const int nb = log - zs_highbit(x);
        tab[i] = zs_cell(s, (uint32_t)nb, (x << nb) - size);
    }
    return true;
}

// Normalized counts from a forward bit stream at src[0, n): returns the bytes
// used, or -1.  max_log bounds the accuracy, *nsym the symbols.
ZS_HD int64_t zs_read_ncount(const uint8_t *src, int64_t n, int max_log, int max_sym, int16_t *norm, int *nsym,
                             int *log) {
    int64_t pos = 0;  // bit position
    if (n < 1) return -1;
    const int al = (int)zs_bits(src, n, pos, 4) + 5;
    pos += 4;
    if (al > max_log) return -1;
    *log = al;
    int32_t remaining = (1 << al) + 1, threshold = 1 << al;
    int nbits = al + 1, s = 0;
    while (remaining > 1) {
        if (s >= max_sym || (pos >> 3) >= n) return -1;
        const int32_t maxv = 2 * threshold - 1 - remaining;
        int32_t v;
        if ((int32_t)zs_bits(src, n, pos, nbits - 1) < maxv) {
            v = (int32_t)zs_bits(src, n, pos, nbits - 1);
            pos += nbits - 1;
        } else {
            v = (int32_t)zs_bits(src, n, pos, nbits);
            pos += nbits;
            if (v >= threshold) v -= maxv;
        }
        const int32_t cnt = v - 1;
        norm[s++] = (int16_t)cnt;
        remaining -= cnt < 0 ? -cnt : cnt;
        if (cnt == 0) {  // runs of zero counts: 2-bit repeat flags
            for (;;) {
                const uint32_t rep = zs_bits(src, n, pos, 2);
                pos += 2;
                for (uint32_t k = 0; k < rep; k++) {
                    if (s >= max_sym) return -1;
                    norm[s++] = 0;
                }
                if (rep != 3) break;
                if ((pos >> 3) >= n) return -1;
            }
        }
        while (remaining < threshold && nbits > 1) {
            nbits--;
            threshold >>= 1;
        }
    }
    if (remaining != 1) return -1;
    *nsym = s;
    const int64_t used = (pos + 7) >> 3;
    return used <= n ? used : -1;
}

// The predefined distributions of the format.
ZS_HD const int16_t *zs_predef(int which, int *nsym, int *log) {
    static const int16_t LL[36] = {4, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 1, 1, 1, 2, 2,
                                   2, 2, 2, 2, 2, 2, 2, 3, 2, 1, 1, 1, 1, 1, -1, -1, -1, -1};
    static const int16_t ML[53] = {1, 4, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                   1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                                   1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1};
    static const int16_t OF[29] = {1, 1, 1, 1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1,
                                   1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1};
    if (which == 0) {
        *nsym = 36;
        *log = 6;
        return LL;
    }
    if (which == 1) {
        *nsym = 29;
        *log = 5;
        return OF;
    }
    *nsym = 53;
    *log = 6;
    return ML;
}

ZS_HD void zs_ll(uint32_t code, uint32_t *base, int *bits) {
    static const uint32_t B[36] = {0,  1,  2,  3,  4,  5,   6,   7,   8,    9,    10,   11,   12,
                                   13, 14, 15, 16, 18, 20,  22,  24,  28,   32,   40,   48,   64,
                                   128, 256, 512, 1024, 2048, 4096, 8192, 16384, 32768, 65536};
    static const uint8_t N[36] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,  0,  1,  1,
                                  1, 1, 2, 2, 3, 3, 4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16};
    *base = B[code];
    *bits = N[code];
}

ZS_HD void zs_ml(uint32_t code, uint32_t *base, int *bits) {
    static const uint32_t B[53] = {3,  4,  5,  6,  7,  8,  9,  10, 11, 12, 13,  14,  15,   16,   17,   18,   19,   20,
                                   21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31,  32,  33,   34,   35,   37,   39,   41,
                                   43, 47, 51, 59, 67, 83, 99, 131, 259, 515, 1027, 2051, 4099, 8195, 16387, 32771, 65539};
    static const uint8_t N[53] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
                                  0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 3, 3, 4, 4, 5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16};
    *base = B[code];
    *bits = N[code];
}

// A sequence table from its mode: 0 predefined, 1 RLE, 2 described here, 3
// the previous one.  Returns the bytes used, or -1.
ZS_COLD int64_t zs_seq_table(int mode, int which, const uint8_t *src, int64_t n, uint32_t *tab, uint32_t *xtab,
                             int *log, int max_log, int max_sym, bool *have) {
    int16_t norm[64];
    int nsym, al;
    int64_t used;
    if (mode == 0) {
        const int16_t *p = zs_predef(which, &nsym, &al);
        for (int s = 0; s < nsym; s++) norm[s] = p[s];
        if (!zs_fse_build(tab, al, norm, nsym)) return -1;
        used = 0;
    } else if (mode == 1) {
        if (n < 1 || src[0] >= max_sym) return -1;
        tab[0] = zs_cell(src[0], 0, 0);
        al = 0;
        used = 1;
    } else if (mode == 2) {
        used = zs_read_ncount(src, n, max_log, max_sym, norm, &nsym, &al);
        if (used < 0 || !zs_fse_build(tab, al, norm, nsym)) return -1;
    } else {
        return *have ? 0 : -1;  // repeat: the previous block's table
    }
    *log = al;
    *have = true;
    if (xtab) {  // literal / match lengths: each cell's baseline and extra bits
        for (uint32_t i = 0; i < (1u << al); i++) {
            uint32_t base;
            int bits;
            if (which == 0) zs_ll(tab[i] & 0xffu, &base, &bits);
            else zs_ml(tab[i] & 0xffu, &base, &bits);
            xtab[i] = base | ((uint32_t)bits << 24);
        }
    }
    return used;
}

// The Huffman table of a literals section: returns the bytes of its
// description, or -1.
ZS_COLD int64_t zs_huf_table(const uint8_t *src, int64_t n, ZsScratch &S, int *maxbits) {
    if (n < 1) return -1;
    uint8_t w[256];
    int nw = 0;
    int64_t used;
    const uint32_t h = src[0];
    if (h < 128) {  // FSE-compressed weights: h bytes
        if (1 + (int64_t)h > n) return -1;
        int16_t norm[64];
        int nsym, al;
        const int64_t nc = zs_read_ncount(src + 1, h, 6, 16, norm, &nsym, &al);
        if (nc < 0 || !zs_fse_build(S.wt, al, norm, nsym)) return -1;
        ZsBack b;
        if (!zs_back_init(b, src + 1 + nc, (int64_t)h - nc)) return -1;
        uint32_t s1 = zs_read(b, al), s2 = zs_read(b, al);
        for (;;) {
            if (nw >= 255) return -1;
            uint32_t c = S.wt[s1];
            w[nw++] = (uint8_t)(c & 0xff);
            s1 = (c >> 16) + zs_read(b, (int)((c >> 8) & 0xff));
            if (b.pos < 0) {
                if (nw >= 255) return -1;
                w[nw++] = (uint8_t)(S.wt[s2] & 0xff);
                break;
            }
            if (nw >= 255) return -1;
            c = S.wt[s2];
            w[nw++] = (uint8_t)(c & 0xff);
            s2 = (c >> 16) + zs_read(b, (int)((c >> 8) & 0xff));
            if (b.pos < 0) {
                if (nw >= 255) return -1;
                w[nw++] = (uint8_t)(S.wt[s1] & 0xff);
                break;
            }
        }
        used = 1 + h;
    } else {  // direct: 4 bits per weight
        nw = (int)h - 127;
        used = 1 + (nw + 1) / 2;
        if (used > n) return -1;
        for (int i = 0; i < nw; i++) w[i] = (uint8_t)((src[1 + i / 2] >> ((i & 1) ? 0 : 4)) & 15);
    }
    // the last weight completes the sum of 2^(w-1) to a power of two
    uint32_t total = 0;
    for (int i = 0; i < nw; i++) {
        if (w[i] > ZS_HUF_LOG) return -1;
        if (w[i]) total += 1u << (w[i] - 1);
    }
    if (total == 0) return -1;
    const int mb = zs_highbit(total) + 1;
    if (mb > (int)ZS_HUF_LOG) return -1;
    const uint32_t rest = (1u << mb) - total;
    if (rest & (rest - 1)) return -1;  // not a power of two
    w[nw++] = (uint8_t)(zs_highbit(rest) + 1);
    // codes: lower weights (longer codes) first, equal weights in symbol order
    uint32_t start[ZS_HUF_LOG + 2];
    uint32_t cur = 0;
    for (int wt = 1; wt <= mb; wt++) {
        start[wt] = cur;
        for (int i = 0; i < nw; i++)
            if (w[i] == wt) cur += 1u << (wt - 1);
    }
    if (cur != (1u << mb)) return -1;
    for (int i = 0; i < nw; i++) {
        if (!w[i]) continue;
        const uint32_t len = 1u << (w[i] - 1);
        const uint16_t e = (uint16_t)((i << 8) | (mb + 1 - w[i]));
        for (uint32_t k = 0; k < len; k++) S.huf[start[w[i]] + k] = e;
        start[w[i]] += len;
    }
    *maxbits = mb;
    return used;
}

ZS_COLD bool zs_huf_stream(const uint8_t *src, int64_t n, const ZsScratch &S, int mb, uint8_t *out, int64_t count) {
    ZsBack b;
    if (!zs_back_init(b, src, n)) return false;
    for (int64_t i = 0; i < count; i++) {
        const uint16_t e = S.huf[zs_peek(b, mb)];
        out[i] = (uint8_t)(e >> 8);
        b.pos -= e & 0xff;
    }
    return b.pos == 0;
}

// d[0, n) = s[0, n) copied forward.  The bytes are loaded 8 at a time
// before they are stored (one memory round trip per 8 bytes instead of per
// byte) when a chunk cannot read what it writes: no overlap, or a source at
// least 8 bytes behind (`gap`), or a source ahead of the destination (the
// literals, gap 8).  An overlapping match closer than 8 bytes repeats its
// first `gap` bytes, loaded once.
ZS_HD void zs_copy(uint8_t *d, const uint8_t *s, int32_t n, int32_t gap) {
    if (gap >= 8 || gap >= n) {
        for (int32_t i = 0; i < n; i += 8) {
            const int32_t m = n - i < 8 ? n - i : 8;
            uint8_t t[8];
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (k < m) t[k] = s[i + k];
#pragma unroll
            for (int k = 0; k < 8; k++)
                if (k < m) d[i + k] = t[k];
        }
        return;
    }
    uint8_t t[8];
    for (int32_t k = 0; k < gap; k++) t[k] = s[k];
    for (int32_t i = 0, r = 0; i < n; i++) {
        d[i] = t[r];
        r = r + 1 == gap ? 0 : r + 1;
    }
}

// The state a frame carries from block to block.
struct ZsFrame {
    int huf_bits;  // 0: no Huffman table yet
    int ll_log, ml_log, of_log;
    bool have_ll, have_ml, have_of;
    uint32_t rep[3];
};

// One compressed block src[0, n) appended to dst at *op (capacity cap).
ZS_HD bool zs_block(const uint8_t *src, int64_t n, uint8_t *dst, int32_t cap, int32_t *op, ZsScratch &S, ZsFrame &F) {
    // literals section
    if (n < 1) return false;
    const uint32_t b0 = src[0], ltype = b0 & 3, sf = (b0 >> 2) & 3;
    int64_t pos, csize = 0;
    int32_t lsize;
    if (ltype < 2) {
        if (sf == 0 || sf == 2) {
            lsize = (int32_t)(b0 >> 3);
            pos = 1;
        } else if (sf == 1) {
            if (n < 2) return false;
            lsize = (int32_t)((b0 >> 4) + ((uint32_t)src[1] << 4));
            pos = 2;
        } else {
            if (n < 3) return false;
            lsize = (int32_t)((b0 >> 4) + ((uint32_t)src[1] << 4) + ((uint32_t)src[2] << 12));
            pos = 3;
        }
    } else {
        const int hb = sf < 2 ? 3 : (sf == 2 ? 4 : 5);
        if (n < hb) return false;
        uint64_t v = 0;
        for (int k = 0; k < hb; k++) v |= (uint64_t)src[k] << (8 * k);
        const int bits = sf < 2 ? 10 : (sf == 2 ? 14 : 18);
        lsize = (int32_t)((v >> 4) & ((1ull << bits) - 1));
        csize = (int64_t)((v >> (4 + bits)) & ((1ull << bits) - 1));
        pos = hb;
    }
    if (lsize > (int32_t)ZS_BLOCK_MAX || lsize > cap - *op) return false;
    // raw literals are read where they lie in the frame (src and dst are
    // different buffers); the others are decoded into the end of dst
    uint8_t *lbuf = dst + (cap - lsize);
    const uint8_t *lit = lbuf;
    if (ltype == 0) {
        if (pos + lsize > n) return false;
        lit = src + pos;
        pos += lsize;
    } else if (ltype == 1) {
        if (pos + 1 > n) return false;
        for (int32_t i = 0; i < lsize; i++) lbuf[i] = src[pos];
        pos += 1;
    } else {
        if (pos + csize > n) return false;
        const uint8_t *c = src + pos;
        int64_t cn = csize;
        if (ltype == 2) {
            int mb;
            const int64_t used = zs_huf_table(c, cn, S, &mb);
            if (used < 0) return false;
            F.huf_bits = mb;
            c += used;
            cn -= used;
        } else if (!F.huf_bits) {
            return false;  // treeless without an earlier table
        }
        const bool four = sf != 0;
        if (!four) {
            if (!zs_huf_stream(c, cn, S, F.huf_bits, lbuf, lsize)) return false;
        } else {
            if (cn < 6) return false;
            const int64_t s1 = c[0] | (c[1] << 8), s2 = c[2] | (c[3] << 8), s3 = c[4] | (c[5] << 8);
            const int64_t s4 = cn - 6 - s1 - s2 - s3;
            if (s4 < 0) return false;
            const int64_t seg = (lsize + 3) / 4;
            if (3 * seg > lsize) return false;
            const uint8_t *p = c + 6;
            if (!zs_huf_stream(p, s1, S, F.huf_bits, lbuf, seg) ||
                !zs_huf_stream(p + s1, s2, S, F.huf_bits, lbuf + seg, seg) ||
                !zs_huf_stream(p + s1 + s2, s3, S, F.huf_bits, lbuf + 2 * seg, seg) ||
                !zs_huf_stream(p + s1 + s2 + s3, s4, S, F.huf_bits, lbuf + 3 * seg, lsize - 3 * seg))
                return false;
        }
        pos += csize;
    }
    // sequences section
    if (pos >= n) return false;
    int64_t nseq = src[pos];
    if (nseq < 128) {
        pos += 1;
    } else if (nseq < 255) {
        if (pos + 2 > n) return false;
        nseq = ((nseq - 128) << 8) + src[pos + 1];
        pos += 2;
    } else {
        if (pos + 3 > n) return false;
        nseq = src[pos + 1] + ((int64_t)src[pos + 2] << 8) + 0x7F00;
        pos += 3;
    }
    int32_t lp = 0;  // literals copied so far
    if (nseq > 0) {
        if (pos >= n) return false;
        const uint32_t modes = src[pos++];
        if (modes & 3) return false;
        int64_t u;
        if ((u = zs_seq_table((modes >> 6) & 3, 0, src + pos, n - pos, S.ll, S.llx, &F.ll_log, ZS_LL_LOG, 36, &F.have_ll)) < 0)
            return false;
        pos += u;
        if ((u = zs_seq_table((modes >> 4) & 3, 1, src + pos, n - pos, S.of, nullptr, &F.of_log, ZS_OF_LOG, 32, &F.have_of)) < 0)
            return false;
        pos += u;
        if ((u = zs_seq_table((modes >> 2) & 3, 2, src + pos, n - pos, S.ml, S.mlx, &F.ml_log, ZS_ML_LOG, 53, &F.have_ml)) < 0)
            return false;
        pos += u;
        ZsBack b;
        if (!zs_back_init(b, src + pos, n - pos)) return false;
        uint32_t sll = zs_read(b, F.ll_log), sof = zs_read(b, F.of_log), sml = zs_read(b, F.ml_log);
        for (int64_t q = 0; q < nseq; q++) {
            const uint32_t cl = S.ll[sll], co = S.of[sof], cm = S.ml[sml];
            const uint32_t xl = S.llx[sll], xm = S.mlx[sml];
            const uint32_t ofc = co & 0xff;
            if (ofc > 31) return false;
            // offset bits first, then match length, then literal length
            uint32_t ofv = (1u << ofc) + (ofc ? zs_read(b, (int)ofc) : 0u);
            const uint32_t ml = (xm & 0xffffffu) + zs_read(b, (int)(xm >> 24));
            const uint32_t ll = (xl & 0xffffffu) + zs_read(b, (int)(xl >> 24));
            uint32_t off;
            if (ofv > 3) {
                off = ofv - 3;
                F.rep[2] = F.rep[1];
                F.rep[1] = F.rep[0];
                F.rep[0] = off;
            } else {
                const uint32_t idx = ll == 0 ? ofv : ofv - 1;  // 0..3
                if (idx == 0) {
                    off = F.rep[0];
                } else {
                    off = idx == 3 ? F.rep[0] - 1 : F.rep[idx];
                    if (idx >= 2) F.rep[2] = F.rep[1];
                    F.rep[1] = F.rep[0];
                    F.rep[0] = off;
                }
            }
            if (q + 1 < nseq) {  // literal length, match length, offset states
                sll = (cl >> 16) + zs_read(b, (int)((cl >> 8) & 0xff));
                sml = (cm >> 16) + zs_read(b, (int)((cm >> 8) & 0xff));
                sof = (co >> 16) + zs_read(b, (int)((co >> 8) & 0xff));
            }
            if (b.pos < 0) return false;
            // execute: ll literals, then ml bytes from off back
            // ll <= lsize - lp and ll + ml <= cap - op (< 2^31) before op + ll is formed
            if (ll > (uint32_t)(lsize - lp) || ll + ml > (uint32_t)(cap - *op) || off == 0 || off > (uint32_t)*op + ll)
                return false;
            zs_copy(dst + *op, lit + lp, (int32_t)ll, 8);  // forward: never ahead of the literal read
            *op += (int32_t)ll;
            lp += (int32_t)ll;
            zs_copy(dst + *op, dst + *op - off, (int32_t)ml, (int32_t)off);
            *op += (int32_t)ml;
        }
        if (b.pos != 0) return false;
    } else if (pos != n) {
        return false;
    }
    // the remaining literals
    if (lsize - lp > cap - *op) return false;
    for (int32_t i = lp; i < lsize; i++) dst[(*op)++] = lit[i];
    return true;
}

// Decompress the frames of src[0, n) into dst (capacity cap): the bytes
// written, or -1 for a malformed or oversized frame.
ZS_HD int64_t zstd_decompress(const uint8_t *src, int64_t n, uint8_t *dst, int64_t cap64, ZsScratch &S) {
    // output positions are 32-bit: a page holds less than 2 GB
    const int32_t cap = cap64 > 0x7fffffff ? 0x7fffffff : (int32_t)cap64;
    int64_t ip = 0;
    int32_t op = 0;
    while (ip < n) {
        if (n - ip < 4) return -1;
        const uint32_t magic = src[ip] | (src[ip + 1] << 8) | (src[ip + 2] << 16) | ((uint32_t)src[ip + 3] << 24);
        ip += 4;
        if ((magic & 0xFFFFFFF0u) == 0x184D2A50u) {  // skippable frame
            if (n - ip < 4) return -1;
            const int64_t sz = src[ip] | (src[ip + 1] << 8) | (src[ip + 2] << 16) | ((int64_t)src[ip + 3] << 24);
            ip += 4;
            if (sz > n - ip) return -1;
            ip += sz;
            continue;
        }
        if (magic != 0xFD2FB528u) return -1;
        if (ip >= n) return -1;
        const uint32_t fhd = src[ip++];
        const uint32_t fcs_flag = fhd >> 6, single = (fhd >> 5) & 1, checksum = (fhd >> 2) & 1, did = fhd & 3;
        if (fhd & 8) return -1;  // reserved bit
        if (!single) ip += 1;    // window descriptor (the whole page is the window)
        const int dbytes = did == 0 ? 0 : (did == 1 ? 1 : (did == 2 ? 2 : 4));
        if (ip + dbytes > n) return -1;
        for (int k = 0; k < dbytes; k++)
            if (src[ip + k]) return -1;  // a frame that needs a dictionary: not a Parquet page
        ip += dbytes;
        ip += fcs_flag == 0 ? (single ? 1 : 0) : (fcs_flag == 1 ? 2 : (fcs_flag == 2 ? 4 : 8));
        if (ip > n) return -1;
        ZsFrame F;
        F.huf_bits = 0;
        F.ll_log = F.ml_log = F.of_log = 0;
        F.have_ll = F.have_ml = F.have_of = false;
        F.rep[0] = 1;
        F.rep[1] = 4;
        F.rep[2] = 8;
        for (;;) {
            if (n - ip < 3) return -1;
            const uint32_t bh = src[ip] | (src[ip + 1] << 8) | (src[ip + 2] << 16);
            ip += 3;
            const uint32_t last = bh & 1, type = (bh >> 1) & 3;
            const int64_t bsize = bh >> 3;
            if (type == 0) {  // raw
                if (bsize > n - ip || bsize > cap - op) return -1;
                zs_copy(dst + op, src + ip, (int32_t)bsize, 8);
                ip += bsize;
                op += (int32_t)bsize;
            } else if (type == 1) {  // RLE: one byte, bsize times
                if (ip >= n || bsize > cap - op) return -1;
                for (int32_t i = 0; i < (int32_t)bsize; i++) dst[op + i] = src[ip];
                ip += 1;
                op += (int32_t)bsize;
            } else if (type == 2) {
                if (bsize > n - ip || bsize > ZS_BLOCK_MAX) return -1;
                if (!zs_block(src + ip, bsize, dst, cap, &op, S, F)) return -1;
                ip += bsize;
            } else {
                return -1;
            }
            if (last) break;
        }
        if (checksum) {
            if (n - ip < 4) return -1;
            ip += 4;
        }
    }
    return op;
}

}  // namespace gbz
