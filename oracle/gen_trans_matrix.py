"""Generate the HEVC 32x32 inverse-transform matrix (oracle/hevc_trans_matrix.inc)
from the standard's integer cosine coefficients.

Row k, column n approximates 64*sqrt(2)*cos((2n+1) k pi / 64) with the
published integer sets per transform size: 64; 83, 36; 89, 75, 50, 18;
90, 87, 80, 70, 57, 43, 25, 9; and the 16 odd-row values of the 32-point
transform.  Run: python oracle/gen_trans_matrix.py > oracle/hevc_trans_matrix.inc
"""
C = {
    4: [64],                                   # cos(j pi / 4), j = 1
    8: [83, 36],                               # cos(j pi / 8), j = 1, 3
    16: [89, 75, 50, 18],                      # cos(j pi / 16), j odd
    32: [90, 87, 80, 70, 57, 43, 25, 9],       # cos(j pi / 32), j odd
    64: [90, 90, 88, 85, 82, 78, 73, 67, 61, 54, 46, 38, 31, 22, 13, 4],  # cos(j pi / 64), j odd
}


def entry(k: int, n: int) -> int:
    if k == 0:
        return 64
    e = (k & -k).bit_length() - 1        # k = 2^e * o
    o = k >> e
    den = 64 >> e                          # angle (2n+1) o pi / den
    j = ((2 * n + 1) * o) % (2 * den)
    if j > den:
        j = 2 * den - j                    # cos(2 pi - a) = cos(a)
    sign = 1
    if j > den // 2:
        j = den - j                        # cos(pi - a) = -cos(a)
        sign = -1
    return sign * C[den][(j - 1) // 2]


def matrix():
    return [[entry(k, n) for n in range(32)] for k in range(32)]


if __name__ == "__main__":
    for row in matrix():
        print("    {" + ", ".join(str(v) for v in row) + "},")
