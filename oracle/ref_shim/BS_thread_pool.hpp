// Stand-in for BS::thread_pool, written for this repository so the reference's CPU
// solvers compile from their own sources: the reference vendors the real pool as a git
// submodule (external/thread-pool) that is not checked out. The reference uses exactly
// one call, pool.submit_blocks(first, last, block).wait() (source/detail/parallel.h:21),
// where block(begin, end) handles one contiguous slice of [first, last).
//
// TEST INFRASTRUCTURE ONLY: part of the oracle build (oracle/build_oracle.py).
#pragma once
#include <algorithm>
#include <cstddef>
#include <thread>
#include <vector>

namespace BS
{
    class thread_pool
    {
    public:
        explicit thread_pool(std::size_t threads = 0)
            : _threads(threads ? threads : std::max<std::size_t>(1, std::thread::hardware_concurrency()))
        {}

        [[nodiscard]] std::size_t get_thread_count() const { return _threads; }

        class blocks_done
        {
        public:
            void wait() const {}
        };

        // Runs every block before returning; wait() is then a no-op. Blocks are split as
        // evenly as possible, the first (n % blocks) getting one extra element.
        template <typename T, typename F>
        blocks_done submit_blocks(const T first, const T last, F&& block, std::size_t num_blocks = 0)
        {
            if (last <= first)
                return {};
            const std::size_t n = static_cast<std::size_t>(last - first);
            std::size_t blocks = num_blocks ? num_blocks : _threads;
            blocks = std::min(blocks, n);
            const std::size_t base = n / blocks, rem = n % blocks;
            std::vector<std::thread> workers;
            workers.reserve(blocks);
            T at = first;
            T first_begin = first, first_end = first;
            for (std::size_t b = 0; b < blocks; ++b)
            {
                const T len = static_cast<T>(base + (b < rem ? 1 : 0));
                const T begin = at, end = static_cast<T>(at + len);
                at = end;
                if (b == 0)
                {
                    first_begin = begin;
                    first_end = end;
                    continue;
                }
                workers.emplace_back([&block, begin, end] { block(begin, end); });
            }
            block(first_begin, first_end);
            for (std::thread& w : workers)
                w.join();
            return {};
        }

    private:
        std::size_t _threads;
    };
}
