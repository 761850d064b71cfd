/* Host driver of the tangent contraction of the row assembly (row_wt_entry,
   row_block_accum and skew_entry in element.cuh, with their transposed
   operand layouts) for
   tests/test_contraction_host.py: reads one case (nen, corner slots, pressure
   flag, D 15x15, the 5x16 basis table, the three corner vectors and the
   scale) from argv[1], forms every block (a, b) of the element matrix the way
   the row assembly does, row a after row a, in double and in float, and
   writes both element matrices (9 nen^2 values each, block layout
   (a nen + b) 9 + 3i + j, as double) to argv[2]. */
#include <cmath>
#include <cstdio>
#include <vector>

#include "../biofem-ia_gb300/csrc/element.cuh"

using namespace biofem;

template <class R>
static void run(const double *Din, const double *tabin, int nen, const int cs[3], bool pres, const double *vvin,
                double sc, double *out)
{
  std::vector<R> D(225), tabT(16 * kRowPad, R(0)), wT(9 * kRowPad, R(0)), ke((size_t)9 * nen * nen, R(NAN));
  for (int i = 0; i < 225; i++) D[i] = (R)Din[i];
  for (int s = 0; s < 5; s++)
    for (int b = 0; b < 16; b++) tabT[kRowPad * b + s] = (R)tabin[16 * s + b];
  R vv[3][3];
  for (int k = 0; k < 3; k++)
    for (int d = 0; d < 3; d++) vv[k][d] = (R)vvin[3 * k + d];
  for (int a = 0; a < nen; a++) {
    for (int t = 0; t < 45; t++) {
      int pos = -1;
      const R v = row_wt_entry(D.data(), tabT.data() + kRowPad * a, t, &pos);
      wT[pos] = v;
    }
    const bool acorner = pres && (a == cs[0] || a == cs[1] || a == cs[2]);
    for (int b = 0; b < nen; b++)
      for (int q = 0; q < 9; q++) {
        R v = row_block_accum(wT.data() + kRowPad * q, tabT.data() + kRowPad * b, R(0));
        if (acorner)
          for (int k = 0; k < 3; k++)
            if (b == cs[k]) v += skew_entry(q / 3, q % 3, vv[k], (R)sc);
        ke[((size_t)a * nen + b) * 9 + q] = v;
      }
  }
  for (size_t i = 0; i < ke.size(); i++) out[i] = (double)ke[i];
}

int main(int argc, char **argv)
{
  if (argc != 3) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int hdr[5];
  double D[225], tab[80], vv[9], sc;
  const bool ok = std::fread(hdr, sizeof(int), 5, f) == 5 && std::fread(D, sizeof(double), 225, f) == 225 &&
                  std::fread(tab, sizeof(double), 80, f) == 80 && std::fread(vv, sizeof(double), 9, f) == 9 &&
                  std::fread(&sc, sizeof(double), 1, f) == 1;
  std::fclose(f);
  if (!ok) return 4;
  const int nen = hdr[0], cs[3] = {hdr[1], hdr[2], hdr[3]};
  const bool pres = hdr[4] != 0;
  if (nen < 1 || nen > 16) return 5;
  std::vector<double> o64((size_t)9 * nen * nen), o32(o64.size());
  run<double>(D, tab, nen, cs, pres, vv, sc, o64.data());
  run<float>(D, tab, nen, cs, pres, vv, sc, o32.data());
  FILE *g = std::fopen(argv[2], "wb");
  if (!g) return 6;
  std::fwrite(o64.data(), sizeof(double), o64.size(), g);
  std::fwrite(o32.data(), sizeof(double), o32.size(), g);
  std::fclose(g);
  return 0;
}
