// Partitioner tags of the project's TBB stand-in (see pdpd_pool.h).  They choose how finely
// tbb::parallel_for cuts its range:
//   simple_partitioner   every piece split down to the grain size (TBB's rule);
//   auto_partitioner     (the default) split breadth-first until there are about eight pieces
//                        per thread or no piece can be split, pieces never below the grain;
//   static_partitioner   one piece per thread;
//   affinity_partitioner as auto (the stand-in keeps no cache affinity between loops).
#pragma once

namespace tbb {
struct simple_partitioner {};
struct auto_partitioner {};
struct static_partitioner {};
struct affinity_partitioner {};
}  // namespace tbb
