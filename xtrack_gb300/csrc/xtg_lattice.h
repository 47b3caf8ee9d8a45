// Host-side lattice packer interface (see xtg_lattice.cpp).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/xtrack_gb300.h"
#include "xtg_table.h"

namespace xtg {

struct PackedLattice {
    std::vector<unsigned char> bytes;   // concatenated 16-byte aligned records
    std::vector<int64_t> offsets;       // byte offset of record k; [n] = total
    std::vector<double> flops_fast;     // canonical FP64 FLOPs per element
};

// Checks one raw record against the implemented feature set.
int32_t validate_element(const xtg_element& e, int64_t idx, std::string* why);

// Packs `n` raw records. With `backtrack` the records are emitted in
// reverse element order with the backtracking transformation of each
// element's parameters applied (the kernel then always walks forward).
int32_t pack_lattice(const xtg_element* els, int64_t n, const xtg_config& cfg,
                     bool backtrack, PackedLattice* out, std::string* err);

// Canonical FP64 FLOP count of one packed record for one particle.
double canonical_flops(const unsigned char* rec);

}  // namespace xtg
