// XKCP (SHA3) is not shipped with the reference; SHA3 only feeds the inert
// Merkle verifier (merkle_tree.cpp:369), whose digest is never compared.
// Test infrastructure only.
#include <cstddef>
extern "C" int SHA3_256(unsigned char *, const unsigned char *, size_t) { return 0; }
