/* Stand-in for the empty sparsepp submodule of the reference tree.
 * The reference's scan_xp.cpp includes <sparsepp/spp.h> unconditionally but only
 * uses spp::sparse_hash_set under -DHASH_SPP, which the oracle build never sets. */
#pragma once
#include <unordered_set>
namespace spp {
template <class K> using sparse_hash_set = std::unordered_set<K>;
}
