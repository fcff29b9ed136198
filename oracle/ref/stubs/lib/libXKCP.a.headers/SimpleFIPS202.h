/*
 * Declaration of XKCP's SHA3_256, which the reference includes through
 * my_hhash.h.  XKCP is not shipped with the reference.  The only caller on
 * the Blake3 path is the Merkle "verifier" (merkle_tree.cpp:369), whose
 * digest is never compared with anything, so the test oracle links a
 * definition that leaves the output untouched (oracle/ref/ref_glue.cpp).
 * Part of the test infrastructure only.
 */
#pragma once
#include <stddef.h>
int SHA3_256(unsigned char *output, const unsigned char *input, size_t inputByteLen);
