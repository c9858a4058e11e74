// Lane refill: work items of uneven length (per-voxel fits, Monte Carlo histories)
// stepped one tick at a time, with each lane taking the next item of its block's
// range as soon as its own is done, so lanes do not idle behind the longest item
// of their warp.
#pragma once

namespace pvd {

// Lane refill over a block's item range [r0, r1): each lane steps its item with
// tick(); when it is done (non-zero code) finish(code) completes it and the warp
// takes the next items from the shared-memory counter `next` (one atomic per warp,
// lane offsets from the ballot).  init(v) starts item v and returns 0 to start
// ticking or the final code of an item settled at once.  Every lane of the warp runs
// the loop; it ends when the range is exhausted and no lane is still ticking.  The
// caller guarantees that every item finishes after a bounded number of ticks.
template <class Init, class Tick, class Finish>
__device__ __forceinline__ void refill_loop(long long r0, long long r1, unsigned long long* next, Init init,
                                            Tick tick, Finish finish) {
  const int lane = threadIdx.x & 31;
  bool alive = false, exhausted = r0 >= r1;
  while (true) {
    int fin = 0;
    const unsigned need = __ballot_sync(0xffffffffu, !alive && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if ((need >> lane) & 1u) {
        const long long mine = (long long)base + __popc(need & ((1u << lane) - 1u));
        if (mine < r1) {
          const int info = init(mine);
          if (info == 0)
            alive = true;
          else
            fin = info;  // settled at the start
        }
      }
      if ((long long)base + __popc(need) >= r1) exhausted = true;  // the same for every lane
    }
    if (alive) {
      const int info = tick();
      if (info != 0) {
        alive = false;
        fin = info;
      }
    }
    if (fin != 0) finish(fin);
    if (exhausted && !__any_sync(0xffffffffu, alive)) break;
  }
}

}  // namespace pvd
