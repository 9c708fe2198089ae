// mh_hash.cuh -- spatial-hash insertion and deletion (device side).
//
// Occupied slots of a bucket always form a prefix; a bucket's overflow chain
// (headed by slot 0's `next`) is non-empty only when all four slots are used.
// Insertion into the slots is lock-free: a 64-bit atomicCAS claims the first
// empty slot for the packed key.  Appending to the overflow chain and deleting
// take a per-bucket spin lock whose wait is bounded (MH_ERR_TIMEOUT).
#pragma once
#include "mh_internal.cuh"


__device__ __forceinline__ unsigned long long vload_key(const HSlot *s) {
  return *reinterpret_cast<const volatile unsigned long long *>(&s->key);
}
__device__ __forceinline__ int vload_int(const int *p) { return *reinterpret_cast<const volatile int *>(p); }
__device__ __forceinline__ void vstore_int(int *p, int v) { *reinterpret_cast<volatile int *>(p) = v; }

// HashTable::Alloc (core/hash_table.h:279-286): pop from the block stack.
static __device__ int pop_block(const Dev &d, int x, int y, int z) {
  int idx = atomicSub(&d.ctr->heap_top, 1) - 1;
  if (idx < 0) {
    atomicAdd(&d.ctr->heap_top, 1);
    set_error(d, MH_ERR_CAPACITY);
    atomicAdd(&d.ctr->dropped, 1);
    return -1;
  }
  int ptr = d.heap[idx];
  d.block_pos[ptr] = make_int4(x, y, z, 1);
  atomicMax(&d.ctr->high_water, ptr + 1);
  return ptr;
}

static __device__ bool lock_bucket(const Dev &d, uint32_t b) {
  int spins = 0;
  while (atomicCAS(d.bucket_lock + b, 0, 1) != 0) {
    if (++spins > MH_SPIN_LIMIT) {
      set_error(d, MH_ERR_TIMEOUT);
      return false;
    }
    __nanosleep(64);
  }
  __threadfence();
  return true;
}
static __device__ void unlock_bucket(const Dev &d, uint32_t b) {
  __threadfence();
  atomicExch(d.bucket_lock + b, 0);
}

// HashTable::AllocEntry (core/hash_table.h:96-179), without the drop rule.
static __device__ void hash_insert(const Dev &d, int x, int y, int z) {
  if (!key_in_range(x, y, z)) {
    set_error(d, MH_ERR_INVALID);
    return;
  }
  const unsigned long long k = pack_key(x, y, z);
  const uint32_t b = hash_bucket(x, y, z, d.p.bucket_mask);
  HSlot *s = d.slots + (size_t)b * 4;
#pragma unroll 1
  for (int j = 0; j < 4; ++j) {
    unsigned long long ek = vload_key(s + j);
    if (ek == k) return;
    if (ek == MH_KEY_EMPTY) {
      unsigned long long old = atomicCAS(&s[j].key, MH_KEY_EMPTY, k);
      if (old == MH_KEY_EMPTY) {
        vstore_int(&s[j].ptr, pop_block(d, x, y, z));
        return;
      }
      if (old == k) return;
    }
  }
  // bucket full: overflow chain, appended under the bucket lock
  int n = vload_int(&s[0].next);
  for (uint32_t it = 0; it < d.p.linked_list_size && n >= 0; ++it) {
    if (vload_key(d.overflow + n) == k) return;
    n = vload_int(&d.overflow[n].next);
  }
  if (!lock_bucket(d, b)) return;
  int head = vload_int(&s[0].next);
  n = head;
  uint32_t len = 0;
  bool found = false;
  while (n >= 0 && len <= d.p.linked_list_size) {
    if (vload_key(d.overflow + n) == k) {
      found = true;
      break;
    }
    n = vload_int(&d.overflow[n].next);
    ++len;
  }
  if (!found) {
    if (len >= d.p.linked_list_size) {
      set_error(d, MH_ERR_CAPACITY);
      atomicAdd(&d.ctr->dropped, 1);
    } else {
      int o = atomicSub(&d.ctr->ovf_top, 1) - 1;
      if (o < 0) {
        atomicAdd(&d.ctr->ovf_top, 1);
        set_error(d, MH_ERR_CAPACITY);
        atomicAdd(&d.ctr->dropped, 1);
      } else {
        int e = d.overflow_free[o];
        HSlot *ov = d.overflow + e;
        ov->key = k;
        ov->ptr = pop_block(d, x, y, z);
        ov->next = head;
        __threadfence();
        vstore_int(&s[0].next, e);
      }
    }
  }
  unlock_bucket(d, b);
}

// HashTable::FreeEntry (core/hash_table.h:183-255): remove a key under the
// bucket lock, keeping occupied slots a prefix of the bucket (the chain head
// moves into a freed slot, else the last occupied slot does).  Never fails
// for lock contention.  Returns true if the key was present.
static __device__ bool hash_erase(const Dev &d, int x, int y, int z) {
  const unsigned long long k = pack_key(x, y, z);
  const uint32_t b = hash_bucket(x, y, z, d.p.bucket_mask);
  HSlot *s = d.slots + (size_t)b * 4;
  if (!lock_bucket(d, b)) return false;
  bool ok = false;
  int j = 0, last = -1;
  for (int q = 0; q < 4; ++q) {
    unsigned long long ek = vload_key(s + q);
    if (ek == MH_KEY_EMPTY) break;
    last = q;
    if (ek == k) j = q, ok = true;
  }
  int head = vload_int(&s[0].next);
  if (ok) {
    if (head >= 0) {
      HSlot *h = d.overflow + head;
      s[j].key = h->key;
      s[j].ptr = h->ptr;
      s[0].next = h->next;
      h->key = MH_KEY_EMPTY, h->ptr = -1, h->next = -1;
      stack_push(&d.ctr->ovf_top, d.overflow_free, head);
    } else {
      if (j != last) {
        s[j].key = s[last].key;
        s[j].ptr = s[last].ptr;
      }
      s[last].key = MH_KEY_EMPTY;
      s[last].ptr = -1;
    }
  } else {
    int prev = -1, n = head;
    for (uint32_t it = 0; it <= d.p.linked_list_size && n >= 0; ++it) {
      if (vload_key(d.overflow + n) == k) {
        int nx = d.overflow[n].next;
        if (prev < 0) s[0].next = nx;
        else d.overflow[prev].next = nx;
        d.overflow[n].key = MH_KEY_EMPTY, d.overflow[n].ptr = -1, d.overflow[n].next = -1;
        stack_push(&d.ctr->ovf_top, d.overflow_free, n);
        ok = true;
        break;
      }
      prev = n;
      n = d.overflow[n].next;
    }
  }
  unlock_bucket(d, b);
  return ok;
}

