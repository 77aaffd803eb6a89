// Shared device helpers for the GB300 kernels: warp-ordered hash tables used
// by the bit-exact setup kernels and launch bookkeeping.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define GB_FULL 0xffffffffu

// Launch counter shared by every launcher (host side, gb_runtime.c).
extern "C" void gb_count_launch(int n);
#define GB_COUNT(n) gb_count_launch(n)

__device__ __forceinline__ int gb_lane() { return threadIdx.x & 31; }

// Home slot of a key in a table of cap slots: the multiplicative (Fibonacci)
// hash scaled to [0, cap) by its high bits (for a power of two, the top
// log2(cap) bits).  The low bits of the product would only permute key mod
// cap, and the columns of a row from a structured grid differ by multiples of
// the row and plane strides, so they would share low bits and build long
// probe chains.  Any cap works (probing wraps explicitly).
__device__ __forceinline__ unsigned gb_slot(int key, int cap)
{
   return __umulhi((unsigned) key * 2654435761u, (unsigned) cap);
}

__device__ __forceinline__ unsigned gb_next_slot(unsigned s, int cap) { return s + 1 == (unsigned) cap ? 0u : s + 1; }

// Open-addressing table (linear probing) mapping a non-negative key to its
// position in a per-row list kept in discovery order.  hk[] holds -1 in empty
// slots.
__device__ __forceinline__ int gb_tab_find(const int *hk, const int *hp, int cap, int key)
{
   unsigned s = gb_slot(key, cap);
   for (int probe = 0; probe < cap; probe++)
   {
      int k = hk[s];
      if (k == key) { return hp[s]; }
      if (k < 0) { return -1; }
      s = gb_next_slot(s, cap);
   }
   return -1;
}

// Inserts key -> pos; returns the slot used, or -1 when the table is full.
__device__ __forceinline__ int gb_tab_insert(int *hk, int *hp, int cap, int key, int pos)
{
   unsigned s = gb_slot(key, cap);
   for (int probe = 0; probe < cap; probe++)
   {
      int prev = atomicCAS(&hk[s], -1, key);
      if (prev < 0 || prev == key) { hp[s] = pos; return (int) s; }
      s = gb_next_slot(s, cap);
   }
   return -1;
}

// Warp-cooperative ordered insertion.  Every lane calls it; lanes with
// active=true present a key.  Keys new to the table receive positions
// count, count+1, ... in lane order of their first occurrence, i.e. the order
// in which a sequential loop over the lanes' keys would discover them.
// Returns the key's position (-1 for inactive lanes or overflow), sets
// *created on the lane that created the entry, and raises *overflow when the
// list (listcap) or the table fills up.
__device__ __forceinline__ int gb_warp_insert(int *hk, int *hp, int cap, int *lkeys, int *lslot,
                                              int listcap, int &count, int key, bool active,
                                              bool *created, int *overflow)
{
   const int lane = gb_lane();
   int pos = active ? gb_tab_find(hk, hp, cap, key) : -1;
   bool need = active && pos < 0;
   int mkey = need ? key : -(lane + 2);
   unsigned grp = __match_any_sync(GB_FULL, mkey);
   int leader = __ffs(grp) - 1;
   bool lead = need && leader == lane;
   unsigned newmask = __ballot_sync(GB_FULL, lead);
   if (lead)
   {
      int p = count + __popc(newmask & ((1u << lane) - 1u));
      int slot = p < listcap ? gb_tab_insert(hk, hp, cap, key, p) : -1;
      if (slot >= 0) { lkeys[p] = key; lslot[p] = slot; pos = p; }
      else { *overflow = 1; pos = -1; }
   }
   int lp = __shfl_sync(GB_FULL, pos, leader);
   if (need && !lead) { pos = lp; }
   count += __popc(newmask);
   if (count > listcap) { count = listcap; }
   *created = lead;
   __syncwarp();
   return pos;
}

// Clears the table slots used by the first n entries of a row list.  Slots are
// recorded at insertion, so clearing in parallel cannot break probe chains.
__device__ __forceinline__ void gb_warp_clear(int *hk, const int *lslot, int n)
{
   __syncwarp();
   for (int t = gb_lane(); t < n; t += 32) { hk[lslot[t]] = -1; }
   __syncwarp();
}

// Adds the active lanes' v to init in lane order (lowest lane first), serially,
// so the rounding equals that of a sequential loop; result on all lanes.
__device__ __forceinline__ double gb_warp_ordered_sum(double v, bool active, double init)
{
   unsigned m = __ballot_sync(GB_FULL, active);
   double s = init;
   while (m)
   {
      int l = __ffs(m) - 1;
      m &= m - 1;
      s += __shfl_sync(GB_FULL, v, l);
   }
   return s;
}

// Per-warp scratch slab for one ordered table: hash keys/positions (cap, a
// power of two) plus a list of keys, slots and values (listcap = cap / 2).
struct GbSlab
{
   int    *hk;
   int    *hp;
   int    *lkeys;
   int    *lslot;
   double *lvals;
   int     cap;
   int     listcap;
};

__device__ __forceinline__ GbSlab gb_slab(char *base, int cap, int warp)
{
   // layout per warp: hk[cap] hp[cap] lkeys[cap/2] lslot[cap/2] lvals[cap/2]
   size_t bytes = (size_t) cap * 4 * 2 + (size_t) (cap / 2) * (4 + 4 + 8);
   char *p = base + bytes * (size_t) warp;
   GbSlab s;
   s.cap = cap;
   s.listcap = cap / 2;
   s.hk = (int *) p; p += (size_t) cap * 4;
   s.hp = (int *) p; p += (size_t) cap * 4;
   s.lvals = (double *) p; p += (size_t) (cap / 2) * 8;
   s.lkeys = (int *) p; p += (size_t) (cap / 2) * 4;
   s.lslot = (int *) p;
   return s;
}

static inline size_t gb_slab_bytes(int cap)
{
   return (size_t) cap * 4 * 2 + (size_t) (cap / 2) * (4 + 4 + 8);
}

// ---------------------------------------------------------------------------
// Table used by the tiered setup kernels: the hash (key -> position) and the
// row's key list (for clearing), without values -- values are accumulated in
// the output arrays at row_offset + position.  Layout: hk[cap] hp[cap]
// lkeys[cap/2] lslot[cap/2]  (12 * cap bytes).
// ---------------------------------------------------------------------------
struct GbTab
{
   int *hk, *hp, *lkeys, *lslot;
   int  cap, listcap;
};

__device__ __forceinline__ GbTab gb_tab_at(int *base, int cap)
{
   GbTab t;
   t.cap = cap;
   t.listcap = cap / 2;
   t.hk = base;
   t.hp = base + cap;
   t.lkeys = base + 2 * cap;
   t.lslot = base + 2 * cap + cap / 2;
   return t;
}

#define GB_TAB_INTS(cap) (3 * (cap))

// Fills the hash keys of a table with -1 (warp-cooperative).
__device__ __forceinline__ void gb_tab_init(GbTab &t)
{
   for (int k = gb_lane(); k < t.cap; k += 32) { t.hk[k] = -1; }
   __syncwarp();
}

// Ordered insertion as gb_warp_insert; ovf becomes 1 on every lane when the
// table or the list fills up.
__device__ __forceinline__ int gb_winsert(GbTab &t, int &count, int key, bool active, bool &created, int &ovf)
{
   const int lane = gb_lane();
   int pos = active ? gb_tab_find(t.hk, t.hp, t.cap, key) : -1;
   bool need = active && pos < 0;
   int mkey = need ? key : -(lane + 2);
   unsigned grp = __match_any_sync(GB_FULL, mkey);
   int leader = __ffs(grp) - 1;
   bool lead = need && leader == lane;
   unsigned newmask = __ballot_sync(GB_FULL, lead);
   bool bad = false;
   if (lead)
   {
      int p = count + __popc(newmask & ((1u << lane) - 1u));
      int slot = p < t.listcap ? gb_tab_insert(t.hk, t.hp, t.cap, key, p) : -1;
      if (slot >= 0) { t.lkeys[p] = key; t.lslot[p] = slot; pos = p; }
      else { bad = true; pos = -1; }
   }
   int lp = __shfl_sync(GB_FULL, pos, leader);
   if (need && !lead) { pos = lp; }
   count += __popc(newmask);
   if (count > t.listcap) { count = t.listcap; }
   if (__any_sync(GB_FULL, bad)) { ovf = 1; }
   created = lead;
   __syncwarp();
   return pos;
}

__device__ __forceinline__ void gb_tab_clear(GbTab &t, int n)
{
   __syncwarp();
   if (n > t.listcap) { n = t.listcap; }
   for (int k = gb_lane(); k < n; k += 32) { t.hk[t.lslot[k]] = -1; }
   __syncwarp();
}

// shared-memory tier: 1024-slot table (512 list entries) per warp, 4 warps
#define GB_SMEM_CAP 1024
#define GB_SMEM_WARPS 4
#define GB_SMEM_BYTES (GB_SMEM_WARPS * GB_TAB_INTS(GB_SMEM_CAP) * 4)

// ---------------------------------------------------------------------------
// Compact table for long rows in shared memory: keys (int) and positions
// (16 bit) only, 6 bytes per slot, so more warps fit on an SM.  Without the
// key list the table is cleared by sweeping all slots.  listcap bounds the
// load factor (3/4 of the slots).
// ---------------------------------------------------------------------------
struct GbTabC
{
   int *hk;
   unsigned short *hp;
   int cap, listcap;
};

#define GB_TABC_BYTES(cap) ((cap) * 6)

__device__ __forceinline__ GbTabC gb_tabc_at(char *base, int cap)
{
   GbTabC t;
   t.cap = cap;
   t.listcap = cap / 4 * 3;
   t.hk = (int *) base;
   t.hp = (unsigned short *) (base + (size_t) cap * 4);
   return t;
}

// (compact tables start on 16-byte boundaries and hold a multiple of four
// slots: they are reset with 16-byte stores)
__device__ __forceinline__ void gb_tab_init(GbTabC &t)
{
   const int4 e = make_int4(-1, -1, -1, -1);
   for (int k = 4 * gb_lane(); k < t.cap; k += 128) { *reinterpret_cast<int4 *>(t.hk + k) = e; }
   __syncwarp();
}

__device__ __forceinline__ int gb_tabc_find(const GbTabC &t, int key)
{
   unsigned s = gb_slot(key, t.cap);
   for (int probe = 0; probe < t.cap; probe++)
   {
      int k = t.hk[s];
      if (k == key) { return t.hp[s]; }
      if (k < 0) { return -1; }
      s = gb_next_slot(s, t.cap);
   }
   return -1;
}

__device__ __forceinline__ int gb_tabc_insert(GbTabC &t, int key, int pos)
{
   unsigned s = gb_slot(key, t.cap);
   for (int probe = 0; probe < t.cap; probe++)
   {
      int prev = atomicCAS(&t.hk[s], -1, key);
      if (prev < 0 || prev == key) { t.hp[s] = (unsigned short) pos; return (int) s; }
      s = gb_next_slot(s, t.cap);
   }
   return -1;
}

// Ordered insertion with the semantics of gb_winsert (positions in the order
// of first discovery, lanes in order within a step).
__device__ __forceinline__ int gb_winsert(GbTabC &t, int &count, int key, bool active, bool &created, int &ovf)
{
   const int lane = gb_lane();
   int pos = active ? gb_tabc_find(t, key) : -1;
   bool need = active && pos < 0;
   int mkey = need ? key : -(lane + 2);
   unsigned grp = __match_any_sync(GB_FULL, mkey);
   int leader = __ffs(grp) - 1;
   bool lead = need && leader == lane;
   unsigned newmask = __ballot_sync(GB_FULL, lead);
   bool bad = false;
   if (lead)
   {
      int p = count + __popc(newmask & ((1u << lane) - 1u));
      int slot = p < t.listcap ? gb_tabc_insert(t, key, p) : -1;
      if (slot >= 0) { pos = p; }
      else { bad = true; pos = -1; }
   }
   int lp = __shfl_sync(GB_FULL, pos, leader);
   if (need && !lead) { pos = lp; }
   count += __popc(newmask);
   if (count > t.listcap) { count = t.listcap; }
   if (__any_sync(GB_FULL, bad)) { ovf = 1; }
   created = lead;
   __syncwarp();
   return pos;
}

__device__ __forceinline__ void gb_tab_clear(GbTabC &t, int n)
{
   (void) n;
   __syncwarp();
   const int4 e = make_int4(-1, -1, -1, -1);
   for (int k = 4 * gb_lane(); k < t.cap; k += 128) { *reinterpret_cast<int4 *>(t.hk + k) = e; }
   __syncwarp();
}

// Find / insert on either table type (insert records the slot in GbTab's key
// list so the table can be cleared entry by entry); insert returns false
// when the table is full.
__device__ __forceinline__ int gb_tfind(GbTab &t, int key) { return gb_tab_find(t.hk, t.hp, t.cap, key); }
__device__ __forceinline__ int gb_tfind(GbTabC &t, int key) { return gb_tabc_find(t, key); }
__device__ __forceinline__ bool gb_tinsert(GbTab &t, int key, int p)
{
   int slot = gb_tab_insert(t.hk, t.hp, t.cap, key, p);
   if (slot < 0) { return false; }
   t.lkeys[p] = key;
   t.lslot[p] = slot;
   return true;
}
__device__ __forceinline__ bool gb_tinsert(GbTabC &t, int key, int p) { return gb_tabc_insert(t, key, p) >= 0; }

// Table of a warp in a two-tier kernel: a compact 1024-slot shared-memory
// table (GB_SMEMC_BYTES per block of GB_SMEM_WARPS warps), or a full table in
// global memory for the rows that overflow it.
#define GB_SMEMC_BYTES (GB_SMEM_WARPS * GB_TABC_BYTES(GB_SMEM_CAP))

template <bool GLOBAL> struct GbTierTab { typedef GbTabC type; };
template <> struct GbTierTab<true> { typedef GbTab type; };

template <bool GLOBAL>
__device__ __forceinline__ typename GbTierTab<GLOBAL>::type gb_tier_tab(int *sh, int *gtab, int gcap, int warp)
{
   if constexpr (GLOBAL) { return gb_tab_at(gtab + (size_t) warp * GB_TAB_INTS(gcap), gcap); }
   else { return gb_tabc_at((char *) sh + (threadIdx.x >> 5) * GB_TABC_BYTES(GB_SMEM_CAP), GB_SMEM_CAP); }
}

// ---------------------------------------------------------------------------
// Counting insertion for symbolic passes: only the number of distinct keys
// matters, so each active lane inserts its key directly (one probe sequence
// with atomicCAS) and the new keys are counted with a ballot; no discovery
// order, no positions.  The slots of new keys are recorded in the key list
// (GbTab) so the table can be cleared entry by entry.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int gb_tab_claim(int *hk, int cap, int key, bool &isnew)
{
   unsigned s = gb_slot(key, cap);
   for (int probe = 0; probe < cap; probe++)
   {
      int prev = atomicCAS(&hk[s], -1, key);
      if (prev < 0) { isnew = true; return (int) s; }
      if (prev == key) { isnew = false; return (int) s; }
      s = gb_next_slot(s, cap);
   }
   isnew = false;
   return -1;
}

__device__ __forceinline__ void gb_wcount(GbTab &t, int &count, int key, bool active, int &ovf)
{
   const int lane = gb_lane();
   bool isnew = false, bad = false;
   int slot = -1;
   if (active)
   {
      slot = gb_tab_claim(t.hk, t.cap, key, isnew);
      if (slot < 0) { bad = true; }
   }
   unsigned m = __ballot_sync(GB_FULL, isnew);
   if (isnew)
   {
      int p = count + __popc(m & ((1u << lane) - 1u));
      if (p < t.listcap) { t.lslot[p] = slot; }
      else { bad = true; }
   }
   count += __popc(m);
   if (count > t.listcap) { count = t.listcap; bad = true; }
   if (__any_sync(GB_FULL, bad)) { ovf = 1; }
   __syncwarp();
}

__device__ __forceinline__ void gb_wcount(GbTabC &t, int &count, int key, bool active, int &ovf)
{
   bool isnew = false, bad = false;
   if (active)
   {
      if (gb_tab_claim(t.hk, t.cap, key, isnew) < 0) { bad = true; }
   }
   count += __popc(__ballot_sync(GB_FULL, isnew));
   if (count > t.listcap) { count = t.listcap; bad = true; }
   if (__any_sync(GB_FULL, bad)) { ovf = 1; }
   __syncwarp();
}
