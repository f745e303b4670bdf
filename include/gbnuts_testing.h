/*
 * Test hooks of the gbnuts library.  They have no counterpart in the
 * reference; they exist so the tests can check device building blocks in
 * isolation.
 */
#ifndef GBNUTS_TESTING_H
#define GBNUTS_TESTING_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* The chains-on-M layouts: D1 = A . X^T and D2 = R . X with A and R held in
 * tensor memory (128 lanes x 64 32-bit words each, Aw / Rw, written as given:
 * two bf16 per word) and X a 128x128 bf16 matrix (row-major uint16 bit
 * patterns); D1, D2 128x128 fp32 outputs.  Returns 0 on success. */
int gbnuts_tct_probe(const uint32_t* Aw, const uint16_t* X, const uint32_t* Rw, float* D1,
                     float* D2);

#ifdef __cplusplus
}
#endif
#endif
