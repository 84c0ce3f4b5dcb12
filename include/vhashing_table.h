/*
 * vhashing_table.h - header-only C++ view of a volume's block hash in the
 * shape of vhashing::HashTable (include/vhashing.h:622-826 of
 * E-BAO/Voxel-Hashing-SDF), forwarding to the C ABI in vhsdf.h.
 *
 * Keys are block coordinates (the reference's int3).  The host-callable
 * members map one to one:
 *   AllocKeys(std::vector<Key>)   include/vhashing.h:530-603
 *   find (bulk: pool index or -1) include/vhashing.h:128-131
 *   erase (bulk)                  include/vhashing.h:244-256
 *   clearheap                     include/vhashing.h:80-91
 *   key_heap / heap_counter       include/vhashing.h:43,55,417-425
 * The reference's device-side members - operator[] and find (a device
 * reference into a block value) and Filter / Apply (device functors over
 * the table) - are in vhashing_device.cuh, for kernels the caller compiles
 * with nvcc against the addresses device_table() returns; on the host,
 * block contents move through vh_export_blocks / vh_import_blocks.
 */
#ifndef VHASHING_TABLE_H
#define VHASHING_TABLE_H

#include <cstdint>
#include <vector>

#include "vhsdf.h"

namespace vhashing {

struct BlockKey {
  int x, y, z;
};
static_assert(sizeof(BlockKey) == 3 * sizeof(int32_t), "keys are int32 triples");

class BlockHashTable {
 public:
  /* The block hash of an existing volume (not owned). */
  explicit BlockHashTable(vh_handle *h) : h_(h) {}

  /* Inserts the keys (existing ones are kept) and lists them in the block
   * list, as HashTable::AllocKeys. */
  vh_status AllocKeys(const std::vector<BlockKey> &keys) {
    return status_ = vh_alloc_keys(h_, ptr(keys), (int64_t)keys.size(), VH_MEM_HOST);
  }

  /* Pool index of each key, -1 where absent. */
  std::vector<int> find(const std::vector<BlockKey> &keys) {
    std::vector<int> out(keys.size(), -1);
    if (!keys.empty())
      status_ = vh_find_keys(h_, ptr(keys), (int64_t)keys.size(), out.data(), VH_MEM_HOST);
    return out;
  }

  /* Erases the keys (their blocks are zeroed and recycled); returns how many
   * were present. */
  int64_t erase(const std::vector<BlockKey> &keys) {
    int64_t n = 0;
    status_ = vh_erase_keys(h_, ptr(keys), (int64_t)keys.size(), &n, VH_MEM_HOST);
    return n;
  }

  /* Empties the block list (the reference's key heap). */
  vh_status clearheap() { return status_ = vh_clear_block_list(h_); }

  /* Keys of the block list. */
  std::vector<BlockKey> key_heap() {
    int64_t n = 0;
    status_ = vh_block_list(h_, nullptr, 0, &n);
    std::vector<BlockKey> keys((size_t)n);
    if (status_ == VH_OK && n > 0)
      status_ = vh_block_list(h_, reinterpret_cast<int32_t *>(keys.data()), n, &n);
    return keys;
  }

  int64_t heap_counter() {
    int64_t n = 0;
    status_ = vh_block_list(h_, nullptr, 0, &n);
    return n;
  }

  /* Device addresses of the hash and the block pool for kernels compiled
   * against vhashing_device.cuh (HashTable's device members). */
  vh_device_table device_table() {
    vh_device_table t{};
    status_ = vh_get_device_table(h_, &t);
    return t;
  }

  vh_status last_status() const { return status_; }

 private:
  static const int32_t *ptr(const std::vector<BlockKey> &keys) {
    return reinterpret_cast<const int32_t *>(keys.data());
  }

  vh_handle *h_;
  vh_status status_ = VH_OK;
};

}  // namespace vhashing

#endif  // VHASHING_TABLE_H
