/* Test infrastructure (oracle only): result record shared by the oracle
 * restatement (liboracle.so) and the wrapper over the compiled reference
 * (_ref/libhjref.so).  Each output column is returned as one contiguous host
 * buffer of num_pages * 8192 bytes in the reference page format. */
#ifndef ORACLE_RESULT_H
#define ORACLE_RESULT_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_result {
    int32_t   status;     /* HJ_* status */
    char      error[256]; /* exception message when status != 0 */
    uint64_t  num_rows;
    uint32_t  num_columns;
    int32_t*  types;
    uint64_t* num_pages;
    uint8_t** pages;
} oracle_result;

void oracle_result_free(oracle_result* r);

#ifdef __cplusplus
}
#endif

#endif
