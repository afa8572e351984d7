// (M, V) pairs instantiated per op (fwd, fwddiff, bwd); generated with mg_prop_*.cu
#pragma once
static const int kInst[3][12][2] = {
  {{2, 4}, {2, 8}, {4, 2}, {4, 4}, {4, 8}, {8, 1}, {8, 2}, {8, 4}, {8, 8}, {16, 1}, {16, 2}, {16, 4}},
  {{2, 4}, {4, 2}, {4, 4}, {8, 1}, {8, 2}, {8, 4}, {16, 1}, {16, 2}},
  {{2, 4}, {4, 2}, {4, 4}, {8, 1}, {8, 2}, {8, 4}, {16, 1}, {16, 2}}
};
static const int kInstCount[3] = {12, 8, 8};
