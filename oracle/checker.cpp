// Test infrastructure (oracle only): result checking.
//
//  * oracle_decode_*      restate Table::from_columnar (src/build_table.cpp:513-637
//                         of eleanalt/hash-join-optimizer): pages -> rows.  The
//                         checker decodes GPU and reference pages with this one
//                         reader, independent of the GPU library's own decoder.
//  * oracle_row_hashes    per-row 64-bit fingerprints of decoded columns; the
//                         order-independent checksum of a table is their sum
//                         mod 2^64 and sorted fingerprints give a canonical row
//                         order for tables too large to sort as tuples.
//  * oracle_unchained_*   restate UnchainedHash (include/unchained.h:14-247):
//                         Fibonacci hash of std::hash<int32_t> (sign-extending
//                         identity), next_pow2(n) directory, 4-bit-per-key
//                         16-bit Bloom word, (start << 16 | bloom) entries and a
//                         sentinel (n << 16).
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/hj_api.h"

namespace {

constexpr size_t PAGE = 8192;

inline uint16_t rd16(const uint8_t* p) {
    uint16_t v;
    std::memcpy(&v, p, 2);
    return v;
}

inline uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

inline uint64_t fnv1a(const uint8_t* p, uint64_t n) {
    uint64_t h = 14695981039346656037ull;
    for (uint64_t i = 0; i < n; ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

}  // namespace

extern "C" {

// INT32 pages -> values + validity (0/1 per row).  Returns HJ_ERR_CAPACITY when
// more than cap rows are present (*n_rows = rows needed).
int oracle_decode_int32(const uint8_t* pages, uint64_t n_pages, int32_t* vals, uint8_t* valid,
                        uint64_t cap, uint64_t* n_rows) {
    uint64_t r = 0;
    for (uint64_t p = 0; p < n_pages; ++p) {
        const uint8_t* pg = pages + p * PAGE;
        const uint16_t nr = rd16(pg);
        const uint8_t* bm = pg + PAGE - (nr + 7) / 8;
        uint16_t       d  = 0;
        for (uint16_t i = 0; i < nr; ++i, ++r) {
            if (r >= cap) continue;
            const bool on = bm[i / 8] & (1u << (i % 8));
            valid[r]      = on;
            if (on) std::memcpy(&vals[r], pg + 4 + 4 * size_t(d++), 4);
            else    vals[r] = 0;
        }
    }
    *n_rows = r;
    return r > cap ? HJ_ERR_CAPACITY : HJ_OK;
}

// VARCHAR pages -> (bytes, offsets[n+1], validity).  Long strings (0xffff page
// followed by 0xfffe pages) become one row.  Capacity overflow of rows or bytes
// returns HJ_ERR_CAPACITY with the sizes needed.
int oracle_decode_strings(const uint8_t* pages, uint64_t n_pages, uint8_t* bytes,
                          uint64_t bytes_cap, uint64_t* offsets, uint8_t* valid,
                          uint64_t rows_cap, uint64_t* n_rows, uint64_t* n_bytes) {
    uint64_t r = 0, b = 0;
    bool     over = false;
    auto put = [&](const uint8_t* src, uint64_t len) {
        if (b + len <= bytes_cap) std::memcpy(bytes + b, src, len);
        else                      over = true;
        b += len;
    };
    if (rows_cap > 0) offsets[0] = 0;
    for (uint64_t p = 0; p < n_pages; ++p) {
        const uint8_t* pg = pages + p * PAGE;
        const uint16_t nr = rd16(pg);
        if (nr == 0xffff || nr == 0xfffe) {
            if (nr == 0xffff) {
                if (r < rows_cap) valid[r] = 1;
                ++r;
            }
            put(pg + 4, rd16(pg + 2));
            if (r <= rows_cap) offsets[r] = b;
            continue;
        }
        const uint16_t nn   = rd16(pg + 2);
        const uint8_t* data = pg + 4 + 2 * size_t(nn);
        const uint8_t* bm   = pg + PAGE - (nr + 7) / 8;
        uint16_t       d = 0, start = 0;
        for (uint16_t i = 0; i < nr; ++i) {
            const bool on = bm[i / 8] & (1u << (i % 8));
            if (on) {
                const uint16_t end = rd16(pg + 4 + 2 * size_t(d++));
                put(data + start, uint64_t(end) - start);
                start = end;
            }
            if (r < rows_cap) valid[r] = on;
            ++r;
            if (r <= rows_cap) offsets[r] = b;
        }
    }
    *n_rows  = r;
    *n_bytes = b;
    return (r > rows_cap || over) ? HJ_ERR_CAPACITY : HJ_OK;
}

// Folds one decoded column into per-row fingerprints (call once per column,
// in column order, starting from h[i] = 0).  kind: HJ_INT32 (vals/valid) or
// HJ_VARCHAR (bytes/offsets/valid).
int oracle_row_hashes(uint64_t* h, uint64_t n, uint32_t column, int32_t kind, const int32_t* vals,
                      const uint8_t* bytes, const uint64_t* offsets, const uint8_t* valid) {
    const uint64_t salt = mix64(0x636f6c756d6eull + column);
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t v;
        if (!valid[i])            v = 0x4e554c4c4e554c4cull;  // NULL
        else if (kind == HJ_INT32) v = mix64(0x100000000ull | uint32_t(vals[i]));
        else v = fnv1a(bytes + offsets[i], offsets[i + 1] - offsets[i]) ^ mix64(offsets[i + 1] - offsets[i]);
        h[i] = mix64(h[i] ^ mix64(v ^ salt));
    }
    return HJ_OK;
}

// Sum of fingerprints mod 2^64: the order-independent table checksum.
uint64_t oracle_checksum(const uint64_t* h, uint64_t n) {
    uint64_t s = 0;
    for (uint64_t i = 0; i < n; ++i) s += h[i];
    return s;
}

// UnchainedHash<int32_t, *>::finalize_build directory words (dir_size + 1 of
// them) for build keys `keys`; *dir_size = next_pow2(n) (0 when n == 0).
int oracle_unchained_directory(const int32_t* keys, uint64_t n, uint64_t* dir, uint64_t cap,
                               uint64_t* dir_size) {
    if (n == 0) {
        *dir_size = 0;
        return HJ_OK;
    }
    uint64_t ds = 1;
    while (ds < n) ds <<= 1;
    unsigned bits = 0;
    while ((1ull << bits) < ds) ++bits;
    *dir_size = ds;
    if (ds + 1 > cap) return HJ_ERR_CAPACITY;
    std::vector<uint64_t> counts(ds, 0);
    std::vector<uint16_t> bloom(ds, 0);
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t h = uint64_t(int64_t(keys[i])) * 11400714819323198485ull;
        const uint64_t p = bits == 0 ? 0 : h >> (64 - bits);
        const uint16_t s = uint16_t(h);
        counts[p]++;
        bloom[p] |= uint16_t((1u << (s & 15)) | (1u << ((s >> 4) & 15)) | (1u << ((s >> 8) & 15))
                             | (1u << ((s >> 12) & 15)));
    }
    uint64_t start = 0;
    for (uint64_t p = 0; p < ds; ++p) {
        dir[p] = (start << 16) | bloom[p];
        start += counts[p];
    }
    dir[ds] = start << 16;
    return HJ_OK;
}

// UnchainedHash::probe match counts (Bloom reject, then key compare over the
// bucket range) for each probe key.
int oracle_unchained_counts(const int32_t* build, uint64_t nb, const int32_t* probe, uint64_t np,
                            uint64_t* counts) {
    std::vector<uint64_t> dir(nb == 0 ? 1 : 2 * nb + 2);
    uint64_t              ds = 0;
    oracle_unchained_directory(build, nb, dir.data(), dir.size(), &ds);
    if (ds == 0) {
        for (uint64_t i = 0; i < np; ++i) counts[i] = 0;
        return HJ_OK;
    }
    unsigned bits = 0;
    while ((1ull << bits) < ds) ++bits;
    // adjacency array in bucket order (within-bucket order does not affect counts)
    std::vector<uint64_t> fill(ds, 0);
    std::vector<int32_t>  adj(nb);
    for (uint64_t i = 0; i < nb; ++i) {
        const uint64_t h = uint64_t(int64_t(build[i])) * 11400714819323198485ull;
        const uint64_t p = bits == 0 ? 0 : h >> (64 - bits);
        adj[(dir[p] >> 16) + fill[p]++] = build[i];
    }
    for (uint64_t i = 0; i < np; ++i) {
        const uint64_t h = uint64_t(int64_t(probe[i])) * 11400714819323198485ull;
        const uint64_t p = bits == 0 ? 0 : h >> (64 - bits);
        const uint16_t s = uint16_t(h);
        const uint16_t m = uint16_t((1u << (s & 15)) | (1u << ((s >> 4) & 15))
                                    | (1u << ((s >> 8) & 15)) | (1u << ((s >> 12) & 15)));
        uint64_t c = 0;
        if ((uint16_t(dir[p]) & m) == m)
            for (uint64_t j = dir[p] >> 16; j < (dir[p + 1] >> 16); ++j) c += adj[j] == probe[i];
        counts[i] = c;
    }
    return HJ_OK;
}

}  // extern "C"
