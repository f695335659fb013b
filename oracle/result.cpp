// Test infrastructure (oracle only): frees an oracle_result.
#include "oracle_result.h"

extern "C" void oracle_result_free(oracle_result* r) {
    if (!r) return;
    for (uint32_t c = 0; c < r->num_columns; ++c) delete[] r->pages[c];
    delete[] r->pages;
    delete[] r->types;
    delete[] r->num_pages;
    r->pages       = nullptr;
    r->types       = nullptr;
    r->num_pages   = nullptr;
    r->num_columns = 0;
}
