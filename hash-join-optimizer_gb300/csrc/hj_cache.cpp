// Binary table files: the reference's table cache format (DumpTable,
// include/table.h:128-211, read by Table::from_cache, src/build_table.cpp:
// 147-203), so files written by either side load on the other.
//
// Layout: a TableMeta header {u64 num_rows; u64 num_cols; DataType types[16];
// u64 num_pages[16]} padded with zeros to one 8 KiB page, then every page of
// column 0, of column 1, ... back to back.  Loading maps the file, points the
// columns' pages into the mapping and uploads them to HBM as a resident table
// (with host memory access the GPU reads the mapped pages itself), then
// unmaps: one file read, no per-page host copies.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/hj_api.h"

namespace {

constexpr size_t   kPageBytes = 8192;
constexpr uint32_t kMaxCols   = 16;

struct FileMeta {  // the reference's TableMeta, byte for byte
    uint64_t num_rows;
    uint64_t num_cols;
    int32_t  types[kMaxCols];
    uint64_t num_pages[kMaxCols];
};
static_assert(sizeof(FileMeta) == 208, "TableMeta layout");

}  // namespace

extern "C" {

int hj_table_dump(const hj_table_desc* t, const char* path) {
    if (!t || !path || t->num_columns > kMaxCols || (t->num_columns && !t->columns) || t->resident)
        return HJ_ERR_INVALID;
    FileMeta meta{};
    meta.num_rows = t->num_rows;
    meta.num_cols = t->num_columns;
    for (uint32_t c = 0; c < t->num_columns; ++c) {
        meta.types[c]     = t->columns[c].type;
        meta.num_pages[c] = t->columns[c].num_pages;
        if (t->columns[c].num_pages && !t->columns[c].pages) return HJ_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return HJ_ERR_RUNTIME;
    std::vector<uint8_t> head(kPageBytes, 0);
    std::memcpy(head.data(), &meta, sizeof(meta));
    bool ok = std::fwrite(head.data(), 1, kPageBytes, f) == kPageBytes;
    for (uint32_t c = 0; ok && c < t->num_columns; ++c)
        for (uint64_t p = 0; ok && p < t->columns[c].num_pages; ++p)
            ok = std::fwrite(t->columns[c].pages[p], 1, kPageBytes, f) == kPageBytes;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? HJ_OK : HJ_ERR_RUNTIME;
}

int hj_table_load(hj_context* ctx, const char* path, uint64_t* handle) {
    if (!ctx || !path || !handle) return HJ_ERR_INVALID;
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return HJ_ERR_RUNTIME;
    struct stat sb;
    if (fstat(fd, &sb) != 0 || size_t(sb.st_size) < kPageBytes) {
        close(fd);
        return HJ_ERR_INVALID;
    }
    const size_t size = size_t(sb.st_size);
    int          flags = MAP_PRIVATE;
#ifdef MAP_POPULATE
    flags |= MAP_POPULATE;
#endif
    void* mem = mmap(nullptr, size, PROT_READ, flags, fd, 0);
    close(fd);
    if (mem == MAP_FAILED) return HJ_ERR_RUNTIME;
    FileMeta meta;
    std::memcpy(&meta, mem, sizeof(meta));
    int rc = HJ_OK;
    uint64_t total = 0;
    if (meta.num_cols > kMaxCols) rc = HJ_ERR_INVALID;
    for (uint64_t c = 0; rc == HJ_OK && c < meta.num_cols; ++c) {
        if (meta.types[c] < HJ_INT32 || meta.types[c] > HJ_VARCHAR || meta.num_pages[c] > size / kPageBytes)
            rc = HJ_ERR_INVALID;
        total += meta.num_pages[c];
    }
    if (rc == HJ_OK && kPageBytes * (1 + total) != size) rc = HJ_ERR_INVALID;  // truncated or padded file
    if (rc == HJ_OK) {
        std::vector<hj_column_desc>            cols(meta.num_cols);
        std::vector<std::vector<const void*>> ptrs(meta.num_cols);
        const uint8_t*                        data = static_cast<const uint8_t*>(mem) + kPageBytes;
        for (uint64_t c = 0; c < meta.num_cols; ++c) {
            for (uint64_t p = 0; p < meta.num_pages[c]; ++p) ptrs[c].push_back(data + p * kPageBytes);
            data += meta.num_pages[c] * kPageBytes;
            cols[c] = hj_column_desc{meta.types[c], meta.num_pages[c], ptrs[c].empty() ? nullptr : ptrs[c].data()};
        }
        const hj_table_desc t{meta.num_rows, uint32_t(meta.num_cols), cols.empty() ? nullptr : cols.data(), 0};
        rc = hj_table_upload(ctx, &t, handle);  // synchronous: the mapping is read before it returns
    }
    munmap(mem, size);
    return rc;
}

}  // extern "C"
