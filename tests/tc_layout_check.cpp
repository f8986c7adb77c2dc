// Host check of the tensor-core operand layout and descriptors of nsg_tc.cuh: prints
// the element offsets of the tile shapes the MLP inference uses and the descriptor
// words, for an independent restatement in the test to compare.
#include <cstdio>
#include <initializer_list>

#include "nsg_tc.cuh"

int main()
{
    const unsigned shapes[][2] = {{128, 16}, {128, 64}, {64, 16}, {64, 64}, {16, 64}};
    for (const auto &sh : shapes) {
        std::printf("tile %u %u lbo %u\n", sh[0], sh[1], nsg::tc_lbo(sh[0]));
        for (unsigned row = 0; row < sh[0]; row++)
            for (unsigned k = 0; k < sh[1]; k++) std::printf("%u\n", nsg::tc_offset(sh[0], row, k));
    }
    const unsigned addrs[] = {0, 2048, 10240, 12288, 28672, 227 * 1024 - 16};
    for (unsigned a : addrs)
        for (unsigned lbo : {256u, 1024u, 2048u})
            std::printf("desc %u %u %llu\n", a, lbo, (unsigned long long)nsg::tc_smem_desc(a, lbo, nsg::kTcSbo));
    for (unsigned n : {16u, 64u, 256u}) std::printf("idesc %u %u\n", n, nsg::tc_idesc_bf16(128, n));
    return 0;
}
