// Host check of the mixed pair kernel's work cut (nbg_chunk_start and
// nbg_work_chunk in nbg_internal.cuh): chunk 0 starts at unit 0 and chunk C
// at W, every chunk holds work, and every unit maps to the chunk that holds
// it, including 2^50-unit workloads where c * W would overflow 64 bits.
#include <cstdio>

#include "nbg_internal.cuh"

int main()
{
    long long bad = 0, checked = 0;
    const int Cs[] = {1, 2, 3, 4, 5, 7, 32, 100, 608, 760, 4864, 24320, 29184};
    const long long Ws[] = {1, 5, 2048, 9999, 65536, 123457, 1000003, 67108864, 100663303};
    for (int C : Cs)
        for (long long W : Ws) {
            if (C > 1 && W < 2048LL * C) continue; /* k_begin keeps W >= 2048 C */
            ll prev = -1;
            for (ll c = 0; c <= C; c++) {
                const ll s = nbg_chunk_start(c, C, W);
                if ((c == 0 && s != 0) || (c == C && s != W) || s <= prev) bad++;
                prev = s;
            }
            const ll step = W / 20000 + 1;
            for (ll u = 0; u < W; u += (u % 5 == 0 ? 1 : step)) {
                const int c = nbg_work_chunk(u, C, W);
                checked++;
                if (c < 0 || c >= C || nbg_chunk_start(c, C, W) > u || nbg_chunk_start(c + 1, C, W) <= u) bad++;
            }
            for (ll c = 0; c < C; c++) {
                const ll a = nbg_chunk_start(c, C, W), b = nbg_chunk_start(c + 1, C, W) - 1;
                checked += 2;
                if (nbg_work_chunk(a, C, W) != c || nbg_work_chunk(b, C, W) != c) bad++;
            }
        }
    const ll W = (1LL << 50) + 12345;
    const int C = 29184;
    for (ll c = 0; c <= C; c += 97) {
        const ll s = nbg_chunk_start(c, C, W);
        checked++;
        if (s < 0 || s > W || (c < C && nbg_work_chunk(s, C, W) != c)) bad++;
    }
    printf("checked %lld, bad %lld\n", checked, bad);
    return bad != 0;
}
