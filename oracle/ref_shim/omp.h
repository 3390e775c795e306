// The oracle library is single-threaded per structure; OpenMP pragmas in the
// reference compile away and the thread-count setters are no-ops.
#pragma once
inline void omp_set_num_threads(int) {}
inline int omp_get_max_threads() { return 1; }
inline int omp_get_thread_num() { return 0; }
inline int omp_get_num_threads() { return 1; }
