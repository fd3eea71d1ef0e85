/*
 * animate_oracle.h -- THE ORACLE for the ANIMATE frames.  TEST INFRASTRUCTURE ONLY.  Included by
 * chi2_oracle.c (compiled with -ffp-contract=off).
 *
 * A plain CPU restatement of compute_rgb (cuda.c:2394-2540) for n_frames snapshots given their
 * geometry (orc_model_geometry's 20 doubles per snapshot): the image axes from E, four lines of
 * sight per pixel through its corners (2.4 x 2.4 window), their intersection with the ellipsoid
 * (b, c, 1), the red spot of radius SPOT_RAD = 0.04f around the +b axis, the sunlit / shadow
 * colours of asteroid.h:300-313 accumulated in float, the pixel value int(br / 4.0) clamped to
 * [0, 255], and the reference's slip in the shadow branch (blue accumulates onto green,
 * cuda.c:2523).  Layout rgb[ic + 3*(x + S*(y + S*frame))].
 */
void orc_render(const double* geo, int n_frames, int S, unsigned char* rgb)
{
    const float SMIN_R = 6, SMIN_G = 8, SMIN_B = 10, SMAX_R = 30, SMAX_G = 41, SMAX_B = 53;
    const float IMAX_R = 255, IMAX_G = 191, IMAX_B = 144, SPOT_RAD = 0.04f;
    for (int f = 0; f < n_frames; f++) {
        const double* g = geo + 20 * (int64_t)f;
        const double E_x = g[2], E_y = g[3], E_z = g[4];
        const double scale0 = 1.0 / sqrt(E_x * E_x + E_z * E_z);
        const double Z1x = -E_z * scale0, Z1y = 0.0, Z1z = E_x * scale0;
        const double Y1x = -E_x * E_y * scale0, Y1y = (E_x * E_x + E_z * E_z) * scale0, Y1z = -E_y * E_z * scale0;
        const double b = g[0], c = g[1], Ep_b = g[5], Ep_c = g[6], Ep_a = g[7], Sp_b = g[8], Sp_c = g[9], Sp_a = g[10];
        for (int iz = 0; iz < S; iz++)
            for (int iy = 0; iy < S; iy++) {
                float br[3] = {0, 0, 0};
                for (int jz = 0; jz < 2; jz++) {
                    const double z1 = 2.4 * (double)(iz - S / 2 + jz) / (double)S;
                    for (int jy = 0; jy < 2; jy++) {
                        const double y1 = 2.4 * (double)(iy - S / 2 + jy) / (double)S;
                        const double p_x = y1 * Y1x + z1 * Z1x, p_y = y1 * Y1y + z1 * Z1y, p_z = y1 * Y1z + z1 * Z1z;
                        const double p_b = g[11] * p_x + g[12] * p_y + g[13] * p_z;
                        const double p_c = g[14] * p_x + g[15] * p_y + g[16] * p_z;
                        const double p_a = g[17] * p_x + g[18] * p_y + g[19] * p_z;
                        const double A = Ep_b * Ep_b / (b * b) + Ep_c * Ep_c / (c * c) + Ep_a * Ep_a;
                        const double B = 2.0 * (p_b * Ep_b / (b * b) + p_c * Ep_c / (c * c) + p_a * Ep_a);
                        const double C = p_b * p_b / (b * b) + p_c * p_c / (c * c) + p_a * p_a - 1.0;
                        const double D = B * B - 4.0 * A * C;
                        if (!(D >= 0.0)) continue;
                        double lambda = (-B - sqrt(D)) / (2.0 * A);
                        const double lambda1 = (-B + sqrt(D)) / (2.0 * A);
                        if (lambda1 > lambda) lambda = lambda1;
                        const double ri_b = p_b + lambda * Ep_b, ri_c = p_c + lambda * Ep_c, ri_a = p_a + lambda * Ep_a;
                        const int red_spot = (ri_c * ri_c + ri_a * ri_a < SPOT_RAD * SPOT_RAD && ri_b > 0.0);
                        double ni_b = ri_b / (b * b), ni_c = ri_c / (c * c), ni_a = ri_a;
                        const double scale = 1.0 / sqrt(ni_b * ni_b + ni_c * ni_c + ni_a * ni_a);
                        ni_b = ni_b * scale; ni_c = ni_c * scale; ni_a = ni_a * scale;
                        const double I = ni_b * Sp_b + ni_c * Sp_c + ni_a * Sp_a;
                        if (I >= 0.0) {
                            br[0] = br[0] + SMAX_R + I * (IMAX_R - SMAX_R);
                            if (!red_spot) {
                                br[1] = br[1] + SMAX_G + I * (IMAX_G - SMAX_G);
                                br[2] = br[2] + SMAX_B + I * (IMAX_B - SMAX_B);
                            }
                        } else {
                            br[0] = br[0] + SMAX_R + I * (SMAX_R - SMIN_R);
                            if (!red_spot) {
                                br[1] = br[1] + SMAX_G + I * (SMAX_G - SMIN_G);
                                br[2] = br[1] + SMAX_B + I * (SMAX_B - SMIN_B);
                            }
                        }
                    }
                }
                for (int ic = 0; ic < 3; ic++) {
                    int v = (int)(br[ic] / 4.0);
                    if (v > 255) v = 255;
                    if (v < 0) v = 0;
                    rgb[ic + 3 * ((int64_t)iy + (int64_t)S * ((int64_t)iz + (int64_t)S * f))] = (unsigned char)v;
                }
            }
    }
}
