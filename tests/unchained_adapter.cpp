// The UnchainedHash-shaped adapter (include/hj_unchained.h) used the way the
// reference's probe workers use UnchainedHash (src/execute.cpp:111-165 of
// eleanalt/hash-join-optimizer): build_insert every build tuple,
// finalize_build, then probe(key, cb) per key.  Checked against a brute-force
// multimap for every probe key, and the directory against UnchainedHash's
// construction (include/unchained.h:163-217: next_pow2 directory, counts by
// the top hash bits, prefix sums, OR of Bloom masks) restated here.  Prints
// "ok" on success.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <map>
#include <random>
#include <vector>

#include "hj_unchained.h"

struct Payload {
    int64_t row;
    int32_t tag;
};

static uint64_t fib(int32_t k) { return uint64_t(int64_t(k)) * 11400714819323198485ull; }

static std::vector<uint64_t> unchained_directory(const std::vector<int32_t>& keys) {
    uint32_t n = uint32_t(keys.size()), size = 1, bits = 0;
    while (size < n) size <<= 1, ++bits;
    std::vector<uint32_t> cnt(size, 0);
    std::vector<uint16_t> bloom(size, 0);
    for (int32_t k : keys) {
        const uint64_t h = fib(k);
        const uint32_t p = bits ? uint32_t(h >> (64 - bits)) : 0;
        const uint32_t s = uint32_t(h & 0xffff);
        ++cnt[p];
        bloom[p] |= uint16_t((1u << (s & 15)) | (1u << ((s >> 4) & 15)) | (1u << ((s >> 8) & 15)) | (1u << ((s >> 12) & 15)));
    }
    std::vector<uint64_t> dir(size + 1);
    uint64_t              off = 0;
    for (uint32_t p = 0; p < size; ++p) {
        dir[p] = (off << 16) | bloom[p];
        off += cnt[p];
    }
    dir[size] = off << 16;
    return dir;
}

static int fail(const char* what, size_t n) {
    std::printf("FAIL %s (build size %zu)\n", what, n);
    return 1;
}

int main() {
    hj_context* ctx = hj_context_create(0);
    if (!ctx) return fail("hj_context_create", 0);
    std::mt19937_64 rng(7);
    for (size_t n : {size_t(1), size_t(2), size_t(3), size_t(1000), size_t(65536), size_t(65537), size_t(200000)}) {
        std::vector<int32_t> keys(n);
        std::uniform_int_distribution<int32_t> dist(-int32_t(n / 2) - 3, int32_t(n / 2) + 3);
        for (size_t i = 0; i < n; ++i) keys[i] = dist(rng);
        if (n >= 3) {
            keys[0] = INT_MIN;
            keys[1] = INT_MAX;
            keys[2] = keys[n - 1];  // a duplicate
        }
        hjgb300::UnchainedHash<int32_t, Payload> ht(ctx);
        ht.reserve(uint32_t(n));
        std::multimap<int32_t, int64_t> truth;
        for (size_t i = 0; i < n; ++i) {
            ht.build_insert(keys[i], Payload{int64_t(i), keys[i] ^ 0x5a5a});
            truth.emplace(keys[i], int64_t(i));
        }
        ht.finalize_build();
        if (ht.directory() != unchained_directory(keys)) return fail("directory words", n);

        // probe keys: every build key plus misses, in a shuffled order
        std::vector<int32_t> probe(keys);
        for (size_t i = 0; i < n / 2 + 4; ++i) probe.push_back(dist(rng) * 3 + 1);
        probe.push_back(INT_MIN + 1);
        std::shuffle(probe.begin(), probe.end(), rng);
        std::vector<std::pair<size_t, int64_t>> got, want;
        bool tags_ok = true;
        ht.probe_batch(probe.data(), probe.size(), [&](size_t i, const Payload& p) {
            got.emplace_back(i, p.row);
            tags_ok &= p.tag == (probe[i] ^ 0x5a5a) && keys[size_t(p.row)] == probe[i];
        });
        for (size_t i = 0; i < probe.size(); ++i) {
            auto r = truth.equal_range(probe[i]);
            for (auto it = r.first; it != r.second; ++it) want.emplace_back(i, it->second);
        }
        std::sort(got.begin(), got.end());
        std::sort(want.begin(), want.end());
        if (!tags_ok) return fail("payload of a match", n);
        if (got != want) return fail("probe_batch matches", n);

        // the reference's one-key form on a few keys
        for (size_t i = 0; i < std::min<size_t>(probe.size(), 8); ++i) {
            std::vector<int64_t> rows, exp;
            ht.probe(probe[i], [&](const Payload& p) { rows.push_back(p.row); });
            auto r = truth.equal_range(probe[i]);
            for (auto it = r.first; it != r.second; ++it) exp.push_back(it->second);
            std::sort(rows.begin(), rows.end());
            std::sort(exp.begin(), exp.end());
            if (rows != exp) return fail("probe(key, cb)", n);
        }
    }
    {  // no tuples: every probe misses
        hjgb300::UnchainedHash<int32_t, Payload> ht(ctx);
        ht.finalize_build();
        int calls = 0;
        ht.probe(5, [&](const Payload&) { ++calls; });
        if (calls) return fail("empty table", 0);
    }
    hj_context_destroy(ctx);
    std::printf("ok\n");
    return 0;
}
