// png.cpp -- self-contained PNG reading and writing for the command-line host.
//
// Reading: zlib / DEFLATE decoding written from RFC 1950 / RFC 1951 (stored, fixed and
// dynamic Huffman blocks, canonical codes decoded one bit at a time), PNG scanline
// filters (None, Sub, Up, Average, Paeth) from the PNG specification, colour types 0, 2,
// 3, 4, 6 at bit depths 1-16 (non-interlaced).  Writing: 8-bit RGB with stored DEFLATE
// blocks (no compression), which any PNG reader accepts.
#include "png.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>

namespace sadcli {
namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
    for (uint32_t n = 0; n < 256; ++n) {
        uint32_t c = n;
        for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = true;
}

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xFFFFFFFFu) {
    if (!crc_ready) crc_init();
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return c;
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) {
    return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | uint32_t(p[3]);
}

// --- DEFLATE decoding --------------------------------------------------------------
struct BitReader {
    const uint8_t* data;
    size_t size;
    size_t pos = 0;   // byte
    int bit = 0;      // bit within byte (LSB first)
    int get() {
        if (pos >= size) throw std::runtime_error("truncated DEFLATE stream");
        int b = (data[pos] >> bit) & 1;
        if (++bit == 8) {
            bit = 0;
            ++pos;
        }
        return b;
    }
    uint32_t bits(int n) {  // n bits, first bit read is the least significant
        uint32_t v = 0;
        for (int i = 0; i < n; ++i) v |= uint32_t(get()) << i;
        return v;
    }
    void align() {
        if (bit) {
            bit = 0;
            ++pos;
        }
    }
};

// Canonical Huffman code: per bit length the number of codes, and the symbols ordered by
// (length, symbol value) -- RFC 1951 section 3.2.2.
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    void build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof(count));
        for (int s = 0; s < n; ++s) count[lengths[s]]++;
        count[0] = 0;
        uint16_t offs[16] = {};
        for (int len = 1; len < 16; ++len) offs[len] = offs[len - 1] + count[len - 1];
        symbol.assign(n, 0);
        for (int s = 0; s < n; ++s)
            if (lengths[s]) symbol[offs[lengths[s]]++] = uint16_t(s);
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= br.get();
            int c = count[len];
            if (code - first < c) return symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw std::runtime_error("invalid Huffman code");
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                               2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                                6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
    for (;;) {
        int sym = lit.decode(br);
        if (sym < 256) {
            out.push_back(uint8_t(sym));
        } else if (sym == 256) {
            return;
        } else {
            sym -= 257;
            if (sym >= 29) throw std::runtime_error("invalid length code");
            size_t len = kLenBase[sym] + br.bits(kLenExtra[sym]);
            int ds = dist.decode(br);
            if (ds >= 30) throw std::runtime_error("invalid distance code");
            size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > out.size()) throw std::runtime_error("distance beyond output");
            size_t from = out.size() - d;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

std::vector<uint8_t> zlib_decode(const std::vector<uint8_t>& z) {
    if (z.size() < 2 || (z[0] & 0x0F) != 8 || ((uint32_t(z[0]) << 8) | z[1]) % 31 != 0 || (z[1] & 0x20))
        throw std::runtime_error("bad zlib header");
    BitReader br{z.data() + 2, z.size() - 2};
    std::vector<uint8_t> out;
    int final = 0;
    while (!final) {
        final = br.get();
        int type = int(br.bits(2));
        if (type == 0) {
            br.align();
            if (br.pos + 4 > br.size) throw std::runtime_error("truncated stored block");
            uint32_t len = br.data[br.pos] | (uint32_t(br.data[br.pos + 1]) << 8);
            br.pos += 4;
            if (br.pos + len > br.size) throw std::runtime_error("truncated stored block");
            out.insert(out.end(), br.data + br.pos, br.data + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            inflate_block(br, lit, dist, out);
        } else if (type == 2) {
            int hlit = int(br.bits(5)) + 257, hdist = int(br.bits(5)) + 1, hclen = int(br.bits(4)) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = uint8_t(br.bits(3));
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[320] = {};
            int n = 0;
            while (n < hlit + hdist) {
                int sym = clh.decode(br);
                if (sym < 16) {
                    lens[n++] = uint8_t(sym);
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (n == 0) throw std::runtime_error("repeat with no previous length");
                        val = lens[n - 1];
                        rep = 3 + int(br.bits(2));
                    } else if (sym == 17) {
                        rep = 3 + int(br.bits(3));
                    } else {
                        rep = 11 + int(br.bits(7));
                    }
                    if (n + rep > hlit + hdist) throw std::runtime_error("too many code lengths");
                    while (rep--) lens[n++] = val;
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(br, lit, dist, out);
        } else {
            throw std::runtime_error("invalid DEFLATE block type");
        }
    }
    return out;
}

int paeth(int a, int b, int c) {
    int p = a + b - c;
    int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    v.push_back(uint8_t(x >> 24));
    v.push_back(uint8_t(x >> 16));
    v.push_back(uint8_t(x >> 8));
    v.push_back(uint8_t(x));
}

void put_chunk(std::vector<uint8_t>& png, const char* type, const std::vector<uint8_t>& data) {
    put_be32(png, uint32_t(data.size()));
    size_t start = png.size();
    png.insert(png.end(), type, type + 4);
    png.insert(png.end(), data.begin(), data.end());
    put_be32(png, crc32(png.data() + start, png.size() - start) ^ 0xFFFFFFFFu);
}

}  // namespace

Image8 read_png(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<uint8_t> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (buf.size() < 8 || std::memcmp(buf.data(), sig, 8) != 0) throw std::runtime_error(path + " is not a PNG file");
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte;
    while (pos + 8 <= buf.size()) {
        uint32_t len = be32(&buf[pos]);
        const char* type = reinterpret_cast<const char*>(&buf[pos + 4]);
        if (pos + 12 + size_t(len) > buf.size()) throw std::runtime_error("truncated PNG chunk");
        const uint8_t* data = &buf[pos + 8];
        if (!std::memcmp(type, "IHDR", 4)) {
            w = be32(data);
            h = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(data, data + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), data, data + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + size_t(len);
    }
    if (w == 0 || h == 0 || ctype < 0) throw std::runtime_error("PNG without IHDR");
    if (w > (1u << 24) || h > (1u << 24) || uint64_t(w) * h > (uint64_t(1) << 31))
        throw std::runtime_error("PNG dimensions too large");
    if (interlace) throw std::runtime_error("interlaced PNG is not supported");
    int chans = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
    if (!chans) throw std::runtime_error("unsupported PNG colour type");
    if (depth != 1 && depth != 2 && depth != 4 && depth != 8 && depth != 16)
        throw std::runtime_error("unsupported PNG bit depth");
    std::vector<uint8_t> raw = zlib_decode(idat);
    const size_t bits_pp = size_t(chans) * depth;
    const size_t row_bytes = (size_t(w) * bits_pp + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    if (raw.size() < size_t(h) * (row_bytes + 1)) throw std::runtime_error("PNG image data too short");
    std::vector<uint8_t> cur(row_bytes), prev(row_bytes, 0);
    Image8 img;
    img.width = int(w);
    img.height = int(h);
    img.rgb.resize(size_t(w) * h * 3);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* src = &raw[size_t(y) * (row_bytes + 1)];
        int filter = src[0];
        for (size_t i = 0; i < row_bytes; ++i) {
            int x = src[1 + i];
            int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            switch (filter) {
                case 0: break;
                case 1: x += a; break;
                case 2: x += b; break;
                case 3: x += (a + b) / 2; break;
                case 4: x += paeth(a, b, c); break;
                default: throw std::runtime_error("invalid PNG filter");
            }
            cur[i] = uint8_t(x);
        }
        for (uint32_t x = 0; x < w; ++x) {
            auto sample = [&](int ch) -> int {  // channel value scaled to 8 bits
                size_t bit = (size_t(x) * chans + ch) * depth;
                if (depth == 16) return cur[bit / 8];
                if (depth == 8) return cur[bit / 8];
                int v = (cur[bit / 8] >> (8 - depth - int(bit % 8))) & ((1 << depth) - 1);
                return ctype == 3 ? v : v * 255 / ((1 << depth) - 1);
            };
            uint8_t* o = &img.rgb[(size_t(y) * w + x) * 3];
            if (ctype == 3) {
                int idx = sample(0);
                if (size_t(idx) * 3 + 2 >= plte.size()) throw std::runtime_error("PNG palette index out of range");
                o[0] = plte[idx * 3];
                o[1] = plte[idx * 3 + 1];
                o[2] = plte[idx * 3 + 2];
            } else if (chans <= 2) {
                o[0] = o[1] = o[2] = uint8_t(sample(0));
            } else {
                o[0] = uint8_t(sample(0));
                o[1] = uint8_t(sample(1));
                o[2] = uint8_t(sample(2));
            }
        }
        std::swap(cur, prev);
    }
    img.gray = chans <= 2 && ctype != 3;
    return img;
}

bool write_png(const std::string& path, const uint8_t* rgb, int width, int height) {
    std::vector<uint8_t> raw;
    raw.reserve(size_t(height) * (size_t(width) * 3 + 1));
    for (int y = 0; y < height; ++y) {
        raw.push_back(0);  // filter: none
        raw.insert(raw.end(), rgb + size_t(y) * width * 3, rgb + size_t(y + 1) * width * 3);
    }
    std::vector<uint8_t> z = {0x78, 0x01};
    size_t off = 0;
    do {
        size_t len = std::min<size_t>(65535, raw.size() - off);
        bool last = off + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(uint8_t(len));
        z.push_back(uint8_t(len >> 8));
        z.push_back(uint8_t(~len));
        z.push_back(uint8_t(~len >> 8));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        off += len;
    } while (off < raw.size());
    put_be32(z, adler32(raw.data(), raw.size()));
    std::vector<uint8_t> png = {137, 80, 78, 71, 13, 10, 26, 10};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, uint32_t(width));
    put_be32(ihdr, uint32_t(height));
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
    put_chunk(png, "IHDR", ihdr);
    put_chunk(png, "IDAT", z);
    put_chunk(png, "IEND", {});
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    f.write(reinterpret_cast<const char*>(png.data()), std::streamsize(png.size()));
    return bool(f);
}

}  // namespace sadcli
