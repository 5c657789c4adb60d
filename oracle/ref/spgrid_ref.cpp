// TEST INFRASTRUCTURE — golden-vector generator built against the reference's own SPGrid sources.
//
// Compiled by oracle/Makefile (target `ref`) from Lib/SPGrid/Core/*.cpp where they lie in the
// reference tree; output goes to oracle/_ref/ only. It uses the reference's SPGrid_Mask
// (Linear_Offset, Packed_Add, LinearToCoord) and SPGrid_Page_Map (Set_Page / Get_Blocks) and
// drives them the way MpmSimulationBase::sortParticlesAndPolluteGrid (MpmSimulationBase.cpp:1531-1573)
// and MpmGrid::pollute (MpmGrid.h:153-193) do. int_floor / baseNode (MathTools.h:15-25,
// BSplines.h:16-20) are restated here because their headers need Eigen.
//
// usage: spgrid_ref <4|8> <in.bin> <out.bin>
//   in.bin : int64 n, double dx, n*3 double positions (cast to float for precision 4)
//   out.bin: see write order in main()
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <vector>
#include <SPGrid/Core/SPGrid_Mask.h>
#include <SPGrid/Core/SPGrid_Geometry.h>
#include <SPGrid/Core/SPGrid_Page_Map.h>

template <class T>
static int int_floor_restated(T x)
{
    int i = (int)x;
    return i - (i > x);
}

template <class T, int LOG2>
static int run(const char* in, const char* out)
{
    using Mask = SPGrid::SPGrid_Mask<LOG2, LOG2, 3, 12>;
    FILE* f = fopen(in, "rb");
    if (!f) return 2;
    int64_t n;
    double dxd;
    if (fread(&n, 8, 1, f) != 1 || fread(&dxd, 8, 1, f) != 1) return 3;
    std::vector<double> xin(3 * n);
    if (fread(xin.data(), 8, 3 * n, f) != (size_t)(3 * n)) return 4;
    fclose(f);
    T dx = (T)dxd;
    T one_over_dx = (T)1 / dx;
    constexpr int index_bits = 32 - Mask::block_bits;
    std::vector<int32_t> base(3 * n);
    std::vector<uint64_t> off(n), key(n);
    for (int64_t i = 0; i < n; i++) {
        std::array<int, 3> b;
        for (int a = 0; a < 3; a++) {
            T xs = (T)xin[3 * i + a] * one_over_dx;
            b[a] = int_floor_restated<T>(xs - (T)0.5);
            base[3 * i + a] = b[a];
        }
        off[i] = Mask::Linear_Offset(b);
        key[i] = ((off[i] >> Mask::data_bits) << index_bits) + (uint64_t)i;
    }
    std::vector<uint64_t> sorted(key);
    std::sort(sorted.begin(), sorted.end());
    std::vector<int32_t> order(n), gfirst, glast;
    std::vector<uint64_t> gblock;
    int last = 0;
    for (int64_t i = 0; i < n; i++) {
        if (i == n - 1 || (sorted[i] >> 32) != (sorted[i + 1] >> 32)) {
            gfirst.push_back(last);
            glast.push_back((int32_t)i);
            gblock.push_back(sorted[i] >> 32);
            last = (int)i + 1;
        }
        order[i] = (int32_t)(sorted[i] & ((1ULL << index_bits) - 1));
    }
    // pollute with the reference's page map
    SPGrid::SPGrid_Geometry<3> geom(4096, 4096, 4096, Mask::block_xbits, Mask::block_ybits, Mask::block_zbits);
    SPGrid::SPGrid_Page_Map<12> pm(geom);
    pm.Clear();
    for (int64_t i = 0; i < n; i++) {
        uint64_t o = off[i];
        if (!i || o != off[i - 1]) {
            pm.Set_Page(o);
            int x = 1 << Mask::block_xbits, y = 1 << Mask::block_ybits, z = 1 << Mask::block_zbits;
            for (int a = 0; a <= 1; a++)
                for (int b = 0; b <= 1; b++)
                    for (int c = 0; c <= 1; c++)
                        pm.Set_Page(Mask::Packed_Add(o, Mask::Linear_Offset(x * a, y * b, z * c)));
        }
    }
    pm.Update_Block_Offsets();
    auto blocks = pm.Get_Blocks();
    std::vector<uint64_t> pages(blocks.second);
    for (unsigned q = 0; q < blocks.second; q++) pages[q] = blocks.first[q] >> 12;
    // LinearToCoord round trip and Packed_Add with small signed displacements
    std::vector<int32_t> back(3 * n);
    const int disp[4][3] = { { 1, 0, 0 }, { 0, 2, 1 }, { -1, -1, 2 }, { 2, -2, -1 } };
    std::vector<uint64_t> padd(4 * n);
    for (int64_t i = 0; i < n; i++) {
        auto c = Mask::LinearToCoord(off[i]);
        for (int a = 0; a < 3; a++) back[3 * i + a] = c[a];
        for (int t = 0; t < 4; t++) padd[4 * i + t] = Mask::Packed_Add(off[i], Mask::Linear_Offset(disp[t][0], disp[t][1], disp[t][2]));
    }
    FILE* g = fopen(out, "wb");
    if (!g) return 5;
    uint64_t masks[3] = { (uint64_t)Mask::xmask, (uint64_t)Mask::ymask, (uint64_t)Mask::zmask };
    int32_t bits[5] = { Mask::block_bits, Mask::data_bits, Mask::block_xbits, Mask::block_ybits, Mask::block_zbits };
    int64_t ng = (int64_t)gfirst.size(), np = (int64_t)pages.size();
    fwrite(masks, 8, 3, g);
    fwrite(bits, 4, 5, g);
    fwrite(base.data(), 4, 3 * n, g);
    fwrite(off.data(), 8, n, g);
    fwrite(key.data(), 8, n, g);
    fwrite(sorted.data(), 8, n, g);
    fwrite(order.data(), 4, n, g);
    fwrite(&ng, 8, 1, g);
    fwrite(gfirst.data(), 4, ng, g);
    fwrite(glast.data(), 4, ng, g);
    fwrite(gblock.data(), 8, ng, g);
    fwrite(&np, 8, 1, g);
    fwrite(pages.data(), 8, np, g);
    fwrite(back.data(), 4, 3 * n, g);
    fwrite(padd.data(), 8, 4 * n, g);
    fclose(g);
    return 0;
}

int main(int argc, char** argv)
{
    if (argc != 4) {
        fprintf(stderr, "usage: spgrid_ref <4|8> <in.bin> <out.bin>\n");
        return 1;
    }
    int p = atoi(argv[1]);
    return p == 4 ? run<float, 6>(argv[2], argv[3]) : run<double, 7>(argv[2], argv[3]);
}
