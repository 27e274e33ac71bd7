// Compiled DP se_e2_a network shape and the packed parameter layout shared by the kernels
// and the host packer (matpl_gb300/dp.py: pack_params must produce the same offsets).
#pragma once

namespace matpl {
namespace dp {

constexpr int E = 25;           // embedding width (all three layers)
constexpr int M2 = 16;          // columns of the second descriptor factor
constexpr int DIN = E * M2;     // fitting input = 400
constexpr int F = 50;           // fitting hidden width
constexpr int NA = 4 * E;       // entries of the per-atom descriptor factor A [4][E]

// One embedding net (dp_embedding.py:40-94), widths 1 -> E -> E -> E.
struct EmbOff {
    static constexpr int W0 = 0;                 // [E]       layer 0 weight (1 x E)
    static constexpr int B0 = W0 + E;            // [E]
    static constexpr int W1 = B0 + E;            // [E][E]    (in, out)
    static constexpr int B1 = W1 + E * E;        // [E]
    static constexpr int DT1 = B1 + E;           // [E]       resnet_dt (ones when absent)
    static constexpr int W2 = DT1 + E;           // [E][E]
    static constexpr int B2 = W2 + E * E;        // [E]
    static constexpr int DT2 = B2 + E;           // [E]
    static constexpr int SIZE = DT2 + E;         // 1400
};

// One fitting net (dp_embedding.py:96-163), widths DIN -> F -> F -> F -> 1, plus transposed
// copies of the matrices for the backward pass.
struct FitOff {
    static constexpr int W0 = 0;                 // [DIN][F]
    static constexpr int B0 = W0 + DIN * F;      // [F]
    static constexpr int W1 = B0 + F;            // [F][F]
    static constexpr int B1 = W1 + F * F;        // [F]
    static constexpr int DT1 = B1 + F;           // [F]
    static constexpr int W2 = DT1 + F;           // [F][F]
    static constexpr int B2 = W2 + F * F;        // [F]
    static constexpr int DT2 = B2 + F;           // [F]
    static constexpr int W3 = DT2 + F;           // [F]       last layer (F x 1)
    static constexpr int B3 = W3 + F;            // [1] (+3 pad)
    static constexpr int W0T = B3 + 4;           // [F][DIN]
    static constexpr int W1T = W0T + F * DIN;    // [F][F]
    static constexpr int W2T = W1T + F * F;      // [F][F]
    static constexpr int SIZE = W2T + F * F;
};

inline long long param_count(int ntypes) {
    return (long long)ntypes * ntypes * EmbOff::SIZE + (long long)ntypes * FitOff::SIZE;
}

}  // namespace dp
}  // namespace matpl
