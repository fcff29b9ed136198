// Definitions of the globals that the reference sources declare `extern` and
// that live in translation units the oracle does not compile (main.cpp,
// coPIOP.cpp, New_PCS.cpp).  Values follow the reference's defaults:
// conjectured_security=false (main.cpp:43), whir_k=8 unless a driver sets it
// (Whir.cpp:6).  Test infrastructure only.
#include "config_pc.hpp"
#include "timer.hpp"
#include <unordered_map>
#include <utility>
#include <vector>

using std::pair;
using std::vector;

int MAX_CHUNCK = 0;
double proving_time = 0;
unsigned long int mul_counter = 0;
vector<F> x_transcript, y_transcript;
F current_randomness;
int threads = 1;
vector<vector<pair<int, int>>> A, B, C;

timer vt;
vector<int> whir_sizes;
vector<int> whir_rates;
vector<int> sorted_indexes;
vector<int> sorted_whir_rates;
bool conjectured_security = false;
std::unordered_map<int, int> whir_kappas;

// XKCP is not shipped with the reference; SHA3 only feeds the inert Merkle
// verifier (merkle_tree.cpp:369), whose digest is never compared.
extern "C" int SHA3_256(unsigned char *, const unsigned char *, size_t) { return 0; }
