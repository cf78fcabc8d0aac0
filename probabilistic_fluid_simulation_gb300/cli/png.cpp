// PNG codec of the command-line driver (see png.h). zlib / deflate follow
// RFC 1950 / 1951, PNG the W3C PNG specification (chunks, filters, Adam7).
#include "png.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace pfs {
namespace png {
namespace {

// ---------------------------------------------------------------- checksums
// The table is built once, when first needed, by a function-local static
// (initialisation is thread-safe: frames are encoded on several threads).
struct CrcTable {
    uint32_t t[256];
    CrcTable()
    {
        for (uint32_t n = 0; n < 256; ++n) {
            uint32_t c = n;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
    }
};

uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0)
{
    static const CrcTable table;
    c ^= 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

uint32_t adler32(const uint8_t *p, size_t n)
{
    uint32_t a = 1, b = 0;
    while (n > 0) {
        const size_t k = std::min<size_t>(n, 5552);  // no overflow of b before the reduction
        for (size_t i = 0; i < k; ++i) {
            a += p[i];
            b += a;
        }
        a %= 65521u;
        b %= 65521u;
        p += k;
        n -= k;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t *p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

void put_be32(std::vector<uint8_t> &v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

// ---------------------------------------------------------------- inflate
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

struct BitIn {
    const uint8_t *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;  // bits in buf; below 8 between reads, so they belong to the byte before pos
    bool over = false;
    uint32_t bits(int k)
    {
        while (cnt < k) {
            uint32_t byte = 0;
            if (pos < n) byte = p[pos];
            else over = true;
            ++pos;
            buf |= byte << cnt;
            cnt += 8;
        }
        const uint32_t v = k ? buf & ((1u << k) - 1u) : 0u;
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align()
    {
        buf = 0;
        cnt = 0;
    }
};

// Canonical Huffman code: codes of each length are consecutive and, within a
// length, ordered by symbol; decoding walks the lengths bit by bit.
struct Huffman {
    int16_t count[16];
    int16_t symbol[320];
};

// 0: complete, > 0: incomplete, < 0: over-subscribed.
int huff_build(Huffman &h, const uint8_t *len, int n)
{
    std::memset(h.count, 0, sizeof h.count);
    for (int s = 0; s < n; ++s) h.count[len[s]]++;
    if (h.count[0] == n) return 1;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return -1;
    }
    int offs[16];
    offs[1] = 0;
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    for (int s = 0; s < n; ++s)
        if (len[s]) h.symbol[offs[len[s]]++] = (int16_t)s;
    return left;
}

int huff_decode(BitIn &b, const Huffman &h)
{
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)b.bits(1);
        const int c = h.count[l];
        if (code - c < first) return h.symbol[index + (code - first)];
        index += c;
        first += c;
        first <<= 1;
        code <<= 1;
        if (b.over) return -1;
    }
    return -1;
}

bool inflate_codes(BitIn &b, const Huffman &lit, const Huffman &dist, std::vector<uint8_t> &out, std::string &err)
{
    for (;;) {
        int sym = huff_decode(b, lit);
        if (sym < 0 || b.over) return err = "deflate: bad literal/length code", false;
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return true;
        } else {
            sym -= 257;
            if (sym >= 29) return err = "deflate: bad length symbol", false;
            const size_t len = kLenBase[sym] + b.bits(kLenExtra[sym]);
            const int ds = huff_decode(b, dist);
            if (ds < 0 || ds >= 30) return err = "deflate: bad distance code", false;
            const size_t d = kDistBase[ds] + b.bits(kDistExtra[ds]);
            if (b.over) return err = "deflate: truncated stream", false;
            if (d > out.size()) return err = "deflate: distance beyond the output", false;
            const size_t from = out.size() - d;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);  // may overlap the bytes being written
        }
    }
}

bool inflate_raw(BitIn &b, std::vector<uint8_t> &out, std::string &err)
{
    static Huffman fixed_lit, fixed_dist;
    static bool fixed_ready = false;
    if (!fixed_ready) {
        uint8_t l[288];
        for (int s = 0; s < 144; ++s) l[s] = 8;
        for (int s = 144; s < 256; ++s) l[s] = 9;
        for (int s = 256; s < 280; ++s) l[s] = 7;
        for (int s = 280; s < 288; ++s) l[s] = 8;
        huff_build(fixed_lit, l, 288);
        for (int s = 0; s < 30; ++s) l[s] = 5;
        huff_build(fixed_dist, l, 30);
        fixed_ready = true;
    }
    int last;
    do {
        last = (int)b.bits(1);
        const int type = (int)b.bits(2);
        if (b.over) return err = "deflate: truncated stream", false;
        if (type == 0) {
            b.align();
            if (b.pos + 4 > b.n) return err = "deflate: truncated stored block", false;
            const unsigned len = b.p[b.pos] | (b.p[b.pos + 1] << 8);
            const unsigned nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
            if (len != (~nlen & 0xFFFFu)) return err = "deflate: stored block length check failed", false;
            b.pos += 4;
            if (b.pos + len > b.n) return err = "deflate: truncated stored block", false;
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            if (!inflate_codes(b, fixed_lit, fixed_dist, out, err)) return false;
        } else if (type == 2) {
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            const int nlen = (int)b.bits(5) + 257, ndist = (int)b.bits(5) + 1, ncode = (int)b.bits(4) + 4;
            if (nlen > 286 || ndist > 30) return err = "deflate: bad code counts", false;
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[order[i]] = (uint8_t)b.bits(3);
            Huffman lencode;
            if (huff_build(lencode, cl, 19) != 0) return err = "deflate: bad code-length code", false;
            uint8_t lengths[320] = {0};
            int i = 0;
            while (i < nlen + ndist) {
                const int sym = huff_decode(b, lencode);
                if (sym < 0 || b.over) return err = "deflate: bad code-length symbol", false;
                if (sym < 16) {
                    lengths[i++] = (uint8_t)sym;
                    continue;
                }
                uint8_t val = 0;
                int rep;
                if (sym == 16) {
                    if (i == 0) return err = "deflate: repeat with no previous length", false;
                    val = lengths[i - 1];
                    rep = 3 + (int)b.bits(2);
                } else if (sym == 17) {
                    rep = 3 + (int)b.bits(3);
                } else {
                    rep = 11 + (int)b.bits(7);
                }
                if (i + rep > nlen + ndist) return err = "deflate: too many code lengths", false;
                while (rep--) lengths[i++] = val;
            }
            if (lengths[256] == 0) return err = "deflate: no end-of-block code", false;
            Huffman lit, dist;
            if (huff_build(lit, lengths, nlen) < 0 || huff_build(dist, lengths + nlen, ndist) < 0)
                return err = "deflate: over-subscribed code", false;
            if (!inflate_codes(b, lit, dist, out, err)) return false;
        } else {
            return err = "deflate: reserved block type", false;
        }
    } while (!last);
    b.align();
    return true;
}

// ---------------------------------------------------------------- deflate (fixed codes)
// Bits go out least significant first through a 64-bit accumulator; Huffman
// codes are stored bit-reversed in tables, so every symbol is one put.
struct BitOut {
    std::vector<uint8_t> &v;
    uint64_t buf = 0;
    int cnt = 0;
    explicit BitOut(std::vector<uint8_t> &out) : v(out) {}
    void put(uint32_t value, int n)  // n <= 32
    {
        buf |= (uint64_t)value << cnt;
        cnt += n;
        if (cnt >= 32) {
            for (int k = 0; k < 4; ++k) v.push_back((uint8_t)(buf >> (8 * k)));
            buf >>= 32;
            cnt -= 32;
        }
    }
    void flush()
    {
        while (cnt > 0) {
            v.push_back((uint8_t)buf);
            buf >>= 8;
            cnt -= 8;
        }
        buf = 0;
        cnt = 0;
    }
};

uint32_t reverse_bits(uint32_t code, int n)
{
    uint32_t r = 0;
    for (int k = 0; k < n; ++k) r |= ((code >> k) & 1u) << (n - 1 - k);
    return r;
}

// The fixed literal/length code (RFC 1951 3.2.6), bit-reversed, and for every
// match length 3..258 its code (with the extra bits merged in) and total bit
// count; for distances 1..32768 the same through zlib-style two-level indexing.
struct FixedCodes {
    uint32_t lit[288];
    uint8_t lit_bits[288];
    uint32_t len_code[259];
    uint8_t len_bits[259];
    uint8_t dist_sym[512];
    uint32_t dist_rev[30];  // the 5-bit distance codes, bit-reversed
    FixedCodes()
    {
        for (int j = 0; j < 30; ++j) dist_rev[j] = reverse_bits((uint32_t)j, 5);
        for (int s = 0; s < 288; ++s) {
            uint32_t c;
            int n;
            if (s < 144) c = 0x30 + s, n = 8;
            else if (s < 256) c = 0x190 + (s - 144), n = 9;
            else if (s < 280) c = s - 256, n = 7;
            else c = 0xC0 + (s - 280), n = 8;
            lit[s] = reverse_bits(c, n);
            lit_bits[s] = (uint8_t)n;
        }
        for (int len = 3; len <= 258; ++len) {
            int k = 28;
            while (kLenBase[k] > len) --k;
            const int sym = 257 + k;
            len_code[len] = lit[sym] | ((uint32_t)(len - kLenBase[k]) << lit_bits[sym]);
            len_bits[len] = (uint8_t)(lit_bits[sym] + kLenExtra[k]);
        }
        for (int d = 1; d <= 32768; ++d) {
            int j = 29;
            while (kDistBase[j] > d) --j;
            if (d <= 256) dist_sym[d - 1] = (uint8_t)j;
            else dist_sym[256 + ((d - 1) >> 7)] = (uint8_t)j;
        }
    }
    int dsym(int d) const { return d <= 256 ? dist_sym[d - 1] : dist_sym[256 + ((d - 1) >> 7)]; }
};

const FixedCodes &fixed_codes()
{
    static const FixedCodes c;  // thread-safe one-time initialisation
    return c;
}

// Length of the common prefix of a and b, at most maxlen, 8 bytes at a time.
inline size_t match_len(const uint8_t *a, const uint8_t *b, size_t maxlen)
{
    size_t l = 0;
    while (l + 8 <= maxlen) {
        uint64_t x, y;
        std::memcpy(&x, a + l, 8);
        std::memcpy(&y, b + l, 8);
        const uint64_t z = x ^ y;
        if (z) {
            // first differing byte: the lowest set byte of z on a little-endian host, the highest otherwise
            const uint16_t probe = 1;
            const bool le = *reinterpret_cast<const uint8_t *>(&probe) == 1;
            return l + (size_t)((le ? __builtin_ctzll(z) : __builtin_clzll(z)) >> 3);
        }
        l += 8;
    }
    while (l < maxlen && a[l] == b[l]) ++l;
    return l;
}

// One final block with the fixed codes. Matches come from hash chains over a
// 32 KiB window (3-byte hash): up to kMaxChain candidates per position, the
// search stopping at a match of kNiceLen bytes; every position of a match of
// up to kMaxInsert bytes enters the chains, longer matches insert their first
// and last kMaxInsert positions (long runs repeat themselves, and inserting
// every byte of them made the encoder three times slower).
void deflate_fixed(const uint8_t *d, size_t n, std::vector<uint8_t> &out)
{
    constexpr int kWin = 32768, kHashBits = 15, kMaxChain = 16, kMaxLen = 258, kNiceLen = 128, kMaxInsert = 16;
    const FixedCodes &fc = fixed_codes();
    std::vector<int> head(1 << kHashBits, -1), prev(kWin, -1);
    auto hash = [&](size_t i) {
        return (int)((((uint32_t)d[i] << 16) ^ ((uint32_t)d[i + 1] << 8) ^ d[i + 2]) * 2654435761u >> (32 - kHashBits));
    };
    auto insert = [&](size_t i) {
        if (i + 3 > n) return;
        const int h = hash(i);
        prev[i & (kWin - 1)] = head[h];
        head[h] = (int)i;
    };
    out.reserve(out.size() + n / 4 + 64);
    BitOut o(out);
    o.put(1, 1);  // final block
    o.put(1, 2);  // fixed Huffman codes
    size_t i = 0;
    while (i < n) {
        int best = 0, bestd = 0;
        if (i + 3 <= n) {
            int cand = head[hash(i)];
            const size_t maxlen = std::min<size_t>(kMaxLen, n - i);
            for (int chain = 0; cand >= 0 && chain < kMaxChain; ++chain) {
                const size_t dist = i - (size_t)cand;
                if (dist == 0 || dist > (size_t)kWin - 1) break;
                if (d[cand + best] == d[i + best]) {  // can this candidate beat the best so far?
                    const size_t l = match_len(d + cand, d + i, maxlen);
                    if ((int)l > best) {
                        best = (int)l;
                        bestd = (int)dist;
                        if (l >= (size_t)kNiceLen || l == maxlen) break;
                    }
                }
                const int nxt = prev[cand & (kWin - 1)];
                if (nxt >= cand) break;  // the window slot was reused
                cand = nxt;
            }
        }
        if (best >= 3) {
            o.put(fc.len_code[best], fc.len_bits[best]);
            const int j = fc.dsym(bestd);
            o.put(fc.dist_rev[j] | ((uint32_t)(bestd - kDistBase[j]) << 5), 5 + kDistExtra[j]);
            if (best <= kMaxInsert) {
                for (int k = 0; k < best; ++k) insert(i + k);
            } else {
                for (int k = 0; k < kMaxInsert; ++k) insert(i + k);
                for (int k = best - kMaxInsert; k < best; ++k) insert(i + k);
            }
            i += best;
        } else {
            o.put(fc.lit[d[i]], fc.lit_bits[d[i]]);
            insert(i);
            ++i;
        }
    }
    o.put(fc.lit[256], fc.lit_bits[256]);
    o.flush();
}

// ---------------------------------------------------------------- PNG filters
inline uint8_t paeth(int a, int b, int c)
{
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

bool unfilter_row(int f, uint8_t *row, const uint8_t *prior, size_t stride, int bpp)
{
    switch (f) {
    case 0: return true;
    case 1:
        for (size_t i = bpp; i < stride; ++i) row[i] = (uint8_t)(row[i] + row[i - bpp]);
        return true;
    case 2:
        for (size_t i = 0; i < stride; ++i) row[i] = (uint8_t)(row[i] + prior[i]);
        return true;
    case 3:
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= (size_t)bpp ? row[i - bpp] : 0;
            row[i] = (uint8_t)(row[i] + ((a + prior[i]) >> 1));
        }
        return true;
    case 4:
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= (size_t)bpp ? row[i - bpp] : 0;
            const int c = i >= (size_t)bpp ? prior[i - bpp] : 0;
            row[i] = (uint8_t)(row[i] + paeth(a, prior[i], c));
        }
        return true;
    default: return false;
    }
}

}  // namespace

bool inflate_zlib(const uint8_t *d, size_t n, std::vector<uint8_t> &out, std::string &err)
{
    if (n < 6) return err = "zlib: stream too short", false;
    const unsigned cmf = d[0], flg = d[1];
    if ((cmf & 15u) != 8u || (cmf >> 4) > 7u || ((cmf << 8) | flg) % 31u != 0u)
        return err = "zlib: bad stream header", false;
    if (flg & 0x20u) return err = "zlib: preset dictionaries are not supported", false;
    BitIn b{d + 2, n - 2};
    out.clear();
    if (!inflate_raw(b, out, err)) return false;
    if (b.pos + 4 > b.n) return err = "zlib: missing checksum", false;
    if (be32(b.p + b.pos) != adler32(out.data(), out.size())) return err = "zlib: checksum mismatch", false;
    return true;
}

std::vector<uint8_t> deflate_zlib(const uint8_t *data, size_t size)
{
    std::vector<uint8_t> out = {0x78, 0x01};
    deflate_fixed(data, size, out);
    put_be32(out, adler32(data, size));
    return out;
}

bool decode(const uint8_t *d, size_t n, Image &img, std::string &err)
{
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (n < 8 || std::memcmp(d, sig, 8) != 0) return err = "not a PNG file", false;
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    bool have_ihdr = false, have_iend = false;
    std::vector<uint8_t> idat, plte, trns;
    while (pos + 12 <= n) {
        const uint32_t len = be32(d + pos);
        if (len > n - pos - 12) return err = "PNG chunk runs past the end of the file", false;
        const uint8_t *type = d + pos + 4, *data = d + pos + 8;
        if (crc32(type, 4 + (size_t)len) != be32(data + len)) return err = "PNG chunk CRC mismatch", false;
        const std::string t(reinterpret_cast<const char *>(type), 4);
        if (!have_ihdr && t != "IHDR") return err = "PNG does not start with IHDR", false;
        if (t == "IHDR") {
            if (len != 13) return err = "bad IHDR", false;
            w = be32(data);
            h = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
            if (w == 0 || h == 0 || (uint64_t)w * h > (1ull << 30)) return err = "bad PNG dimensions", false;
            if (data[10] != 0 || data[11] != 0 || interlace > 1) return err = "bad PNG compression/filter/interlace", false;
            const bool ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                            (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                            ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
            if (!ok) return err = "bad PNG colour type / bit depth", false;
            if (depth == 16) return err = "16-bit PNGs are not supported", false;
            have_ihdr = true;
        } else if (t == "PLTE") {
            if (len % 3 || len > 768 || len == 0) return err = "bad PLTE", false;
            plte.assign(data, data + len);
        } else if (t == "tRNS") {
            trns.assign(data, data + len);
        } else if (t == "IDAT") {
            idat.insert(idat.end(), data, data + len);
        } else if (t == "IEND") {
            have_iend = true;
            break;
        } else if ((type[0] & 0x20u) == 0) {
            return err = "unknown critical PNG chunk " + t, false;
        }
        pos += 12 + (size_t)len;
    }
    if (!have_ihdr || !have_iend) return err = "PNG without IHDR or IEND", false;
    if (ctype == 3 && plte.empty()) return err = "palette PNG without PLTE", false;
    std::vector<uint8_t> raw;
    if (!inflate_zlib(idat.data(), idat.size(), raw, err)) return false;

    static const int chans[7] = {1, 0, 3, 1, 2, 0, 4};
    const int bits_pp = chans[ctype] * depth;
    const int bpp = std::max(1, bits_pp / 8);
    img.width = (int)w;
    img.height = (int)h;
    img.rgba.assign((size_t)w * h * 4, 0);
    const int maxv = (1 << depth) - 1;
    auto sample = [&](const uint8_t *row, uint32_t x, int k) -> int {  // channel k of pixel x
        if (depth == 8) return row[(size_t)x * chans[ctype] + k];
        const size_t bit = (size_t)x * depth;  // depth < 8: one channel
        return (row[bit >> 3] >> (8 - depth - (int)(bit & 7))) & maxv;
    };
    static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
    size_t off = 0;
    for (int pass = 0; pass < (interlace ? 7 : 1); ++pass) {
        const uint32_t x0 = interlace ? ax0[pass] : 0, y0 = interlace ? ay0[pass] : 0;
        const uint32_t dx = interlace ? adx[pass] : 1, dy = interlace ? ady[pass] : 1;
        if (x0 >= w || y0 >= h) continue;
        const uint32_t pw = (w - x0 + dx - 1) / dx, ph = (h - y0 + dy - 1) / dy;
        const size_t stride = ((size_t)pw * bits_pp + 7) / 8;
        if (raw.size() - off < (stride + 1) * ph) return err = "PNG image data too short", false;
        std::vector<uint8_t> prior(stride, 0), row(stride);
        for (uint32_t y = 0; y < ph; ++y) {
            const int f = raw[off];
            std::memcpy(row.data(), raw.data() + off + 1, stride);
            off += stride + 1;
            if (!unfilter_row(f, row.data(), prior.data(), stride, bpp)) return err = "bad PNG filter type", false;
            uint8_t *dst = img.rgba.data() + ((size_t)(y0 + y * dy) * w) * 4;
            for (uint32_t x = 0; x < pw; ++x) {
                uint8_t *px = dst + (size_t)(x0 + x * dx) * 4;
                int r, g, b, a = 255;
                if (ctype == 0) {
                    const int v = sample(row.data(), x, 0);
                    if (trns.size() >= 2 && v == ((trns[0] << 8) | trns[1])) a = 0;
                    r = g = b = v * (255 / maxv);
                } else if (ctype == 2) {
                    r = sample(row.data(), x, 0);
                    g = sample(row.data(), x, 1);
                    b = sample(row.data(), x, 2);
                    if (trns.size() >= 6 && r == ((trns[0] << 8) | trns[1]) && g == ((trns[2] << 8) | trns[3]) &&
                        b == ((trns[4] << 8) | trns[5]))
                        a = 0;
                } else if (ctype == 3) {
                    const int k = sample(row.data(), x, 0);
                    if ((size_t)k * 3 >= plte.size()) return err = "PNG palette index out of range", false;
                    r = plte[3 * k];
                    g = plte[3 * k + 1];
                    b = plte[3 * k + 2];
                    if ((size_t)k < trns.size()) a = trns[k];
                } else if (ctype == 4) {
                    r = g = b = sample(row.data(), x, 0);
                    a = sample(row.data(), x, 1);
                } else {
                    r = sample(row.data(), x, 0);
                    g = sample(row.data(), x, 1);
                    b = sample(row.data(), x, 2);
                    a = sample(row.data(), x, 3);
                }
                px[0] = (uint8_t)r;
                px[1] = (uint8_t)g;
                px[2] = (uint8_t)b;
                px[3] = (uint8_t)a;
            }
            std::swap(prior, row);
        }
    }
    return true;
}

// Row filter f of a 4-byte-per-pixel row into out (x - predictor, mod 256),
// returning the sum of the filtered bytes as signed values, |(int8)v|: the
// selection heuristic of the PNG specification. `up` is the previous row
// (all zeros above the first). One straight loop per filter.
long filter_row(int f, const uint8_t *row, const uint8_t *up, size_t stride, uint8_t *out)
{
    long sum = 0;
    auto emit = [&](size_t i, int pred) {
        const uint8_t v = (uint8_t)(row[i] - pred);
        out[i] = v;
        sum += std::abs((int)(int8_t)v);
    };
    const size_t head = std::min<size_t>(4, stride);
    switch (f) {
    case 0:
        for (size_t i = 0; i < stride; ++i) emit(i, 0);
        break;
    case 1:
        for (size_t i = 0; i < head; ++i) emit(i, 0);
        for (size_t i = 4; i < stride; ++i) emit(i, row[i - 4]);
        break;
    case 2:
        for (size_t i = 0; i < stride; ++i) emit(i, up[i]);
        break;
    case 3:
        for (size_t i = 0; i < head; ++i) emit(i, up[i] >> 1);
        for (size_t i = 4; i < stride; ++i) emit(i, (row[i - 4] + up[i]) >> 1);
        break;
    default:
        for (size_t i = 0; i < head; ++i) emit(i, paeth(0, up[i], 0));
        for (size_t i = 4; i < stride; ++i) emit(i, paeth(row[i - 4], up[i], up[i - 4]));
        break;
    }
    return sum;
}

std::vector<uint8_t> encode(const uint8_t *rgba, int width, int height)
{
    const size_t stride = (size_t)width * 4;
    std::vector<uint8_t> filtered((stride + 1) * height);
    std::vector<uint8_t> cand(5 * stride), zero(stride, 0);
    for (int y = 0; y < height; ++y) {
        const uint8_t *row = rgba + (size_t)y * stride;
        const uint8_t *up = y > 0 ? row - stride : zero.data();
        long best_sum = -1;
        int best_f = 0;
        for (int f = 0; f < 5; ++f) {
            const long sum = filter_row(f, row, up, stride, cand.data() + f * stride);
            if (best_sum < 0 || sum < best_sum) {  // the first filter of least sum
                best_sum = sum;
                best_f = f;
            }
        }
        uint8_t *dst = filtered.data() + (size_t)y * (stride + 1);
        dst[0] = (uint8_t)best_f;
        std::memcpy(dst + 1, cand.data() + best_f * stride, stride);
    }
    std::vector<uint8_t> out = {137, 80, 78, 71, 13, 10, 26, 10};
    auto chunk = [&](const char *type, const std::vector<uint8_t> &data) {
        put_be32(out, (uint32_t)data.size());
        const size_t at = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), data.begin(), data.end());
        put_be32(out, crc32(out.data() + at, 4 + data.size()));
    };
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, (uint32_t)width);
    put_be32(ihdr, (uint32_t)height);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    chunk("IHDR", ihdr);
    chunk("IDAT", deflate_zlib(filtered.data(), filtered.size()));
    chunk("IEND", {});
    return out;
}

bool read_file(const std::string &path, Image &out, std::string &err)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return err = "cannot open " + path, false;
    std::vector<uint8_t> data;
    uint8_t buf[1 << 16];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) data.insert(data.end(), buf, buf + k);
    std::fclose(f);
    return decode(data.data(), data.size(), out, err);
}

bool write_file(const std::string &path, const uint8_t *rgba, int width, int height, std::string &err)
{
    const std::vector<uint8_t> data = encode(rgba, width, height);
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return err = "cannot create " + path, false;
    const bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
    if (std::fclose(f) != 0 || !ok) return err = "cannot write " + path, false;
    return true;
}

}  // namespace png
}  // namespace pfs

// C entry points of the codec for the tests (libpfs_png.so). Buffers returned
// through `out` are malloc'd; release them with pfs_png_free.
extern "C" {

int pfs_png_decode(const uint8_t *data, size_t size, uint8_t **out, int *width, int *height, char *err, int errlen)
{
    pfs::png::Image img;
    std::string e;
    if (!pfs::png::decode(data, size, img, e)) {
        if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", e.c_str());
        return 1;
    }
    *out = static_cast<uint8_t *>(std::malloc(img.rgba.size()));
    if (!*out) return 2;
    std::memcpy(*out, img.rgba.data(), img.rgba.size());
    *width = img.width;
    *height = img.height;
    return 0;
}

int pfs_png_encode(const uint8_t *rgba, int width, int height, uint8_t **out, size_t *size)
{
    const std::vector<uint8_t> v = pfs::png::encode(rgba, width, height);
    *out = static_cast<uint8_t *>(std::malloc(v.size()));
    if (!*out) return 2;
    std::memcpy(*out, v.data(), v.size());
    *size = v.size();
    return 0;
}

int pfs_zlib_inflate(const uint8_t *data, size_t size, uint8_t **out, size_t *out_size)
{
    std::vector<uint8_t> v;
    std::string e;
    if (!pfs::png::inflate_zlib(data, size, v, e)) return 1;
    *out = static_cast<uint8_t *>(std::malloc(v.size() ? v.size() : 1));
    if (!*out) return 2;
    if (!v.empty()) std::memcpy(*out, v.data(), v.size());
    *out_size = v.size();
    return 0;
}

void pfs_png_free(void *p) { std::free(p); }

}  // extern "C"
