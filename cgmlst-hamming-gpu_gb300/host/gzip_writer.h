// gzip output stream for the CLI (-z, or -o ending in .gz; main.rs:475-485).
//
// With zlib available at build time (TCH_HAVE_ZLIB) the stream is deflated at
// the requested level (the reference uses level 3).  Without it the writer
// still produces a valid gzip member (RFC 1952) made of stored deflate blocks
// (RFC 1951 BTYPE 00) with its CRC-32 and size trailer: the decompressed
// bytes are identical, only the file is larger.
#pragma once

#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#ifdef TCH_HAVE_ZLIB
#include <zlib.h>
#endif

namespace tch_host {

// CRC-32 (IEEE 802.3, reflected polynomial 0xEDB88320), table driven.
class Crc32 {
   public:
    Crc32() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table_[i] = c;
        }
    }
    void update(const char* p, size_t n) {
        uint32_t c = ~crc_;
        for (size_t i = 0; i < n; i++) c = table_[(c ^ (uint8_t)p[i]) & 0xFF] ^ (c >> 8);
        crc_ = ~c;
    }
    uint32_t value() const { return crc_; }

   private:
    uint32_t table_[256];
    uint32_t crc_ = 0;
};

template <class Out>
class GzipWriter {
   public:
    GzipWriter(Out& out, int level) : out_(out), level_(level) {
#ifdef TCH_HAVE_ZLIB
        memset(&zs_, 0, sizeof zs_);
        ok_ = deflateInit2(&zs_, level_, Z_DEFLATED, 15 + 16, 8, Z_DEFAULT_STRATEGY) == Z_OK;
#else
        static const unsigned char hdr[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 0xff};
        out_.write((const char*)hdr, sizeof hdr);
#endif
    }

    void write(const char* p, size_t n) {
        buf_.append(p, n);
        if (buf_.size() >= (1u << 20)) flush_block(false);
    }

    void finish() { flush_block(true); }

   private:
#ifdef TCH_HAVE_ZLIB
    void flush_block(bool last) {
        std::vector<char> obuf(1 << 20);
        zs_.next_in = (Bytef*)buf_.data();
        zs_.avail_in = (uInt)buf_.size();
        int rc;
        do {
            zs_.next_out = (Bytef*)obuf.data();
            zs_.avail_out = (uInt)obuf.size();
            rc = deflate(&zs_, last ? Z_FINISH : Z_NO_FLUSH);
            out_.write(obuf.data(), obuf.size() - zs_.avail_out);
        } while (zs_.avail_out == 0 || (last && rc != Z_STREAM_END));
        buf_.clear();
        if (last) deflateEnd(&zs_);
    }
    z_stream zs_;
    bool ok_ = false;
#else
    void flush_block(bool last) {
        crc_.update(buf_.data(), buf_.size());
        size_ += buf_.size();
        size_t off = 0;
        do {
            const size_t len = std::min<size_t>(65535, buf_.size() - off);
            const bool final_block = last && off + len == buf_.size();
            unsigned char h[5] = {(unsigned char)(final_block ? 1 : 0), (unsigned char)(len & 0xFF),
                                  (unsigned char)(len >> 8), (unsigned char)(~len & 0xFF),
                                  (unsigned char)((~len >> 8) & 0xFF)};
            out_.write((const char*)h, 5);
            out_.write(buf_.data() + off, len);
            off += len;
        } while (off < buf_.size());
        buf_.clear();
        if (last) {
            unsigned char t[8];
            const uint32_t c = crc_.value(), s = (uint32_t)size_;
            for (int k = 0; k < 4; k++) t[k] = (unsigned char)(c >> (8 * k)), t[4 + k] = (unsigned char)(s >> (8 * k));
            out_.write((const char*)t, 8);
        }
    }
    Crc32 crc_;
    uint64_t size_ = 0;
#endif
    Out& out_;
    int level_;
    std::string buf_;
};

}  // namespace tch_host
