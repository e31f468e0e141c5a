/* Declarations the reference's kem.c relies on implicitly (it is C and includes no header for
 * them); force-included when kem.c is compiled as C++ for the host.  TEST INFRASTRUCTURE ONLY.
 * Definitions: oracle/ref_glue_frodo.cpp. */
#pragma once
#include <stdint.h>
#include "api.h"
#include "frodo_macrify.h"
void frodo_mul_add_as_plus_e(uint16_t *out, const uint16_t *s, const uint16_t *e, const uint8_t *seed_A);
void frodo_mul_add_sa_plus_e(uint16_t *out, const uint16_t *s, const uint16_t *e, const uint8_t *seed_A);
void frodo_mul_add_sb_plus_e(uint16_t *out, const uint16_t *b, const uint16_t *s, const uint16_t *e);
void frodo_mul_bs(uint16_t *out, const uint16_t *b, const uint16_t *s);
void frodo_add(uint16_t *out, const uint16_t *a, const uint16_t *b);
void frodo_sub(uint16_t *out, const uint16_t *a, const uint16_t *b);
void frodo_key_encode(uint16_t *out, const uint16_t *in);
void frodo_key_decode(uint16_t *out, const uint16_t *in);
