// ref_pn_dump START COUNT [THREADS]: prints "n p(n)" for the evens START,
// START + 2, ..., computed by the reference's own CPU fallback
// gb::cpu_min_goldbach_prime (src/primes.cpp:482-493) over the reference's
// candidate list gb::odd_primes_up_to(9781). Linked against the reference's
// src/primes.cpp by oracle/Makefile (target `ref`); used only to generate
// golden fixtures under tests/golden/.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

#include "primes.hpp"

int main(int argc, char** argv)
{
    if (argc < 3) { std::fprintf(stderr, "usage: ref_pn_dump START COUNT [THREADS]\n"); return 2; }
    const uint64_t start = std::strtoull(argv[1], nullptr, 10), count = std::strtoull(argv[2], nullptr, 10);
    const unsigned nt = argc > 3 ? unsigned(std::atoi(argv[3])) : std::max(1u, std::thread::hardware_concurrency());
    const std::vector<uint32_t> pr = gb::odd_primes_up_to(9781);
    std::vector<uint16_t> c16(pr.begin(), pr.end());
    std::vector<uint64_t> out(count);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (uint64_t i = t; i < count; i += nt)
                out[i] = gb::cpu_min_goldbach_prime(start + 2 * i, c16.data(), c16.size(), 9781);
        });
    for (auto& x : th) x.join();
    for (uint64_t i = 0; i < count; ++i)
        std::printf("%llu %llu\n", (unsigned long long)(start + 2 * i), (unsigned long long)out[i]);
    return 0;
}
