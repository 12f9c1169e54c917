// GENERATED by gen_eri.py -- do not edit by hand.
#pragma once

// ---- class (ss|ss): 1x1 integrals, L = 0
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_ssss(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekp00_000 = ONE;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[1];
    boys_eval<T, 0>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    const T hp = T(0.5) * invp;
    {
      const T W_000 = ekp00_000 * R0_000;
      acc[0] += W_000;
    }
  }
}

// ---- class (ps|ss): 3x1 integrals, L = 1
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_psss(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekp00_000 = ONE;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[2];
    boys_eval<T, 1>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T hp = T(0.5) * invp;
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    {
      const T W_000 = ekp00_000 * R0_000;
      const T W_001 = ekp00_000 * R0_001;
      const T W_010 = ekp00_000 * R0_010;
      const T W_100 = ekp00_000 * R0_100;
      acc[0] += fma_t(ebx101, W_100, ebx100 * W_000);
      acc[1] += fma_t(eby101, W_010, eby100 * W_000);
      acc[2] += fma_t(ebz101, W_001, ebz100 * W_000);
    }
  }
}

// ---- class (ps|ps): 3x3 integrals, L = 2
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_psps(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekp00_000 = ekx100;
  const T ekp00_100 = -(ekx101);
  const T ekp10_000 = eky100;
  const T ekp10_010 = -(eky101);
  const T ekp20_000 = ekz100;
  const T ekp20_001 = -(ekz101);
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[3];
    boys_eval<T, 2>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T hp = T(0.5) * invp;
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    {
      const T W_000 = fma_t(ekp00_100, R0_100, ekp00_000 * R0_000);
      const T W_001 = fma_t(ekp00_100, R0_101, ekp00_000 * R0_001);
      const T W_010 = fma_t(ekp00_100, R0_110, ekp00_000 * R0_010);
      const T W_100 = fma_t(ekp00_100, R0_200, ekp00_000 * R0_100);
      acc[0] += fma_t(ebx101, W_100, ebx100 * W_000);
      acc[3] += fma_t(eby101, W_010, eby100 * W_000);
      acc[6] += fma_t(ebz101, W_001, ebz100 * W_000);
    }
    {
      const T W_000 = fma_t(ekp10_010, R0_010, ekp10_000 * R0_000);
      const T W_001 = fma_t(ekp10_010, R0_011, ekp10_000 * R0_001);
      const T W_010 = fma_t(ekp10_010, R0_020, ekp10_000 * R0_010);
      const T W_100 = fma_t(ekp10_010, R0_110, ekp10_000 * R0_100);
      acc[1] += fma_t(ebx101, W_100, ebx100 * W_000);
      acc[4] += fma_t(eby101, W_010, eby100 * W_000);
      acc[7] += fma_t(ebz101, W_001, ebz100 * W_000);
    }
    {
      const T W_000 = fma_t(ekp20_001, R0_001, ekp20_000 * R0_000);
      const T W_001 = fma_t(ekp20_001, R0_002, ekp20_000 * R0_001);
      const T W_010 = fma_t(ekp20_001, R0_011, ekp20_000 * R0_010);
      const T W_100 = fma_t(ekp20_001, R0_101, ekp20_000 * R0_100);
      acc[2] += fma_t(ebx101, W_100, ebx100 * W_000);
      acc[5] += fma_t(eby101, W_010, eby100 * W_000);
      acc[8] += fma_t(ebz101, W_001, ebz100 * W_000);
    }
  }
}

// ---- class (pp|ss): 9x1 integrals, L = 2
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_ppss(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekp00_000 = ONE;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[3];
    boys_eval<T, 2>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T hp = T(0.5) * invp;
    const T ebx010 = PBx;
    const T ebx011 = hp * (ONE);
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx110 = PAx * ebx010 + ebx011;
    const T ebx111 = hp * (ebx010 + ebx100);
    const T ebx112 = (hp * T(0.5)) * (ebx011 + ebx101);
    const T eby010 = PBy;
    const T eby011 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby110 = PAy * eby010 + eby011;
    const T eby111 = hp * (eby010 + eby100);
    const T eby112 = (hp * T(0.5)) * (eby011 + eby101);
    const T ebz010 = PBz;
    const T ebz011 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz110 = PAz * ebz010 + ebz011;
    const T ebz111 = hp * (ebz010 + ebz100);
    const T ebz112 = (hp * T(0.5)) * (ebz011 + ebz101);
    {
      const T W_000 = ekp00_000 * R0_000;
      const T W_001 = ekp00_000 * R0_001;
      const T W_010 = ekp00_000 * R0_010;
      const T W_100 = ekp00_000 * R0_100;
      const T W_002 = ekp00_000 * R0_002;
      const T W_011 = ekp00_000 * R0_011;
      const T W_020 = ekp00_000 * R0_020;
      const T W_101 = ekp00_000 * R0_101;
      const T W_110 = ekp00_000 * R0_110;
      const T W_200 = ekp00_000 * R0_200;
      acc[0] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[1] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[2] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[3] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[4] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[5] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[6] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[7] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[8] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
  }
}

// ---- class (pp|ps): 9x3 integrals, L = 3
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_ppps(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekp00_000 = ekx100;
  const T ekp00_100 = -(ekx101);
  const T ekp10_000 = eky100;
  const T ekp10_010 = -(eky101);
  const T ekp20_000 = ekz100;
  const T ekp20_001 = -(ekz101);
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[4];
    boys_eval<T, 3>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T hp = T(0.5) * invp;
    const T ebx010 = PBx;
    const T ebx011 = hp * (ONE);
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx110 = PAx * ebx010 + ebx011;
    const T ebx111 = hp * (ebx010 + ebx100);
    const T ebx112 = (hp * T(0.5)) * (ebx011 + ebx101);
    const T eby010 = PBy;
    const T eby011 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby110 = PAy * eby010 + eby011;
    const T eby111 = hp * (eby010 + eby100);
    const T eby112 = (hp * T(0.5)) * (eby011 + eby101);
    const T ebz010 = PBz;
    const T ebz011 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz110 = PAz * ebz010 + ebz011;
    const T ebz111 = hp * (ebz010 + ebz100);
    const T ebz112 = (hp * T(0.5)) * (ebz011 + ebz101);
    {
      const T W_000 = fma_t(ekp00_100, R0_100, ekp00_000 * R0_000);
      const T W_001 = fma_t(ekp00_100, R0_101, ekp00_000 * R0_001);
      const T W_010 = fma_t(ekp00_100, R0_110, ekp00_000 * R0_010);
      const T W_100 = fma_t(ekp00_100, R0_200, ekp00_000 * R0_100);
      const T W_002 = fma_t(ekp00_100, R0_102, ekp00_000 * R0_002);
      const T W_011 = fma_t(ekp00_100, R0_111, ekp00_000 * R0_011);
      const T W_020 = fma_t(ekp00_100, R0_120, ekp00_000 * R0_020);
      const T W_101 = fma_t(ekp00_100, R0_201, ekp00_000 * R0_101);
      const T W_110 = fma_t(ekp00_100, R0_210, ekp00_000 * R0_110);
      const T W_200 = fma_t(ekp00_100, R0_300, ekp00_000 * R0_200);
      acc[0] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[3] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[6] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[9] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[12] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[15] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[18] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[21] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[24] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp10_010, R0_010, ekp10_000 * R0_000);
      const T W_001 = fma_t(ekp10_010, R0_011, ekp10_000 * R0_001);
      const T W_010 = fma_t(ekp10_010, R0_020, ekp10_000 * R0_010);
      const T W_100 = fma_t(ekp10_010, R0_110, ekp10_000 * R0_100);
      const T W_002 = fma_t(ekp10_010, R0_012, ekp10_000 * R0_002);
      const T W_011 = fma_t(ekp10_010, R0_021, ekp10_000 * R0_011);
      const T W_020 = fma_t(ekp10_010, R0_030, ekp10_000 * R0_020);
      const T W_101 = fma_t(ekp10_010, R0_111, ekp10_000 * R0_101);
      const T W_110 = fma_t(ekp10_010, R0_120, ekp10_000 * R0_110);
      const T W_200 = fma_t(ekp10_010, R0_210, ekp10_000 * R0_200);
      acc[1] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[4] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[7] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[10] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[13] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[16] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[19] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[22] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[25] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp20_001, R0_001, ekp20_000 * R0_000);
      const T W_001 = fma_t(ekp20_001, R0_002, ekp20_000 * R0_001);
      const T W_010 = fma_t(ekp20_001, R0_011, ekp20_000 * R0_010);
      const T W_100 = fma_t(ekp20_001, R0_101, ekp20_000 * R0_100);
      const T W_002 = fma_t(ekp20_001, R0_003, ekp20_000 * R0_002);
      const T W_011 = fma_t(ekp20_001, R0_012, ekp20_000 * R0_011);
      const T W_020 = fma_t(ekp20_001, R0_021, ekp20_000 * R0_020);
      const T W_101 = fma_t(ekp20_001, R0_102, ekp20_000 * R0_101);
      const T W_110 = fma_t(ekp20_001, R0_111, ekp20_000 * R0_110);
      const T W_200 = fma_t(ekp20_001, R0_201, ekp20_000 * R0_200);
      acc[2] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[5] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[8] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[11] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[14] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[17] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[20] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[23] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[26] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
  }
}

// ---- class (pp|pp): 9x9 integrals, L = 4
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_pppp(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx010 = QDx;
  const T ekx011 = hq * (ONE);
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T ekx110 = QCx * ekx010 + ekx011;
  const T ekx111 = hq * (ekx010 + ekx100);
  const T ekx112 = (hq * T(0.5)) * (ekx011 + ekx101);
  const T eky010 = QDy;
  const T eky011 = hq * (ONE);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T eky110 = QCy * eky010 + eky011;
  const T eky111 = hq * (eky010 + eky100);
  const T eky112 = (hq * T(0.5)) * (eky011 + eky101);
  const T ekz010 = QDz;
  const T ekz011 = hq * (ONE);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekz110 = QCz * ekz010 + ekz011;
  const T ekz111 = hq * (ekz010 + ekz100);
  const T ekz112 = (hq * T(0.5)) * (ekz011 + ekz101);
  const T ekp00_000 = ekx110;
  const T ekp00_100 = -(ekx111);
  const T ekp00_200 = ekx112;
  const T ekp01_000 = ekx100 * eky010;
  const T ekp01_010 = -(ekx100 * eky011);
  const T ekp01_100 = -(ekx101 * eky010);
  const T ekp01_110 = ekx101 * eky011;
  const T ekp02_000 = ekx100 * ekz010;
  const T ekp02_001 = -(ekx100 * ekz011);
  const T ekp02_100 = -(ekx101 * ekz010);
  const T ekp02_101 = ekx101 * ekz011;
  const T ekp10_000 = ekx010 * eky100;
  const T ekp10_010 = -(ekx010 * eky101);
  const T ekp10_100 = -(ekx011 * eky100);
  const T ekp10_110 = ekx011 * eky101;
  const T ekp11_000 = eky110;
  const T ekp11_010 = -(eky111);
  const T ekp11_020 = eky112;
  const T ekp12_000 = eky100 * ekz010;
  const T ekp12_001 = -(eky100 * ekz011);
  const T ekp12_010 = -(eky101 * ekz010);
  const T ekp12_011 = eky101 * ekz011;
  const T ekp20_000 = ekx010 * ekz100;
  const T ekp20_001 = -(ekx010 * ekz101);
  const T ekp20_100 = -(ekx011 * ekz100);
  const T ekp20_101 = ekx011 * ekz101;
  const T ekp21_000 = eky010 * ekz100;
  const T ekp21_001 = -(eky010 * ekz101);
  const T ekp21_010 = -(eky011 * ekz100);
  const T ekp21_011 = eky011 * ekz101;
  const T ekp22_000 = ekz110;
  const T ekp22_001 = -(ekz111);
  const T ekp22_002 = ekz112;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[5];
    boys_eval<T, 4>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    scale *= m2a;
    const T R4_000 = scale * F[4];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T R3_001 = Z * R4_000;
    const T R2_002 = R3_000 + Z * R3_001;
    const T R1_003 = T(2) * R2_001 + Z * R2_002;
    const T R0_004 = T(3) * R1_002 + Z * R1_003;
    const T R0_013 = Y * R1_003;
    const T R1_012 = Y * R2_002;
    const T R0_022 = R1_002 + Y * R1_012;
    const T R2_011 = Y * R3_001;
    const T R1_021 = R2_001 + Y * R2_011;
    const T R0_031 = T(2) * R1_011 + Y * R1_021;
    const T R3_010 = Y * R4_000;
    const T R2_020 = R3_000 + Y * R3_010;
    const T R1_030 = T(2) * R2_010 + Y * R2_020;
    const T R0_040 = T(3) * R1_020 + Y * R1_030;
    const T R0_103 = X * R1_003;
    const T R0_112 = X * R1_012;
    const T R0_121 = X * R1_021;
    const T R0_130 = X * R1_030;
    const T R1_102 = X * R2_002;
    const T R0_202 = R1_002 + X * R1_102;
    const T R1_111 = X * R2_011;
    const T R0_211 = R1_011 + X * R1_111;
    const T R1_120 = X * R2_020;
    const T R0_220 = R1_020 + X * R1_120;
    const T R2_101 = X * R3_001;
    const T R1_201 = R2_001 + X * R2_101;
    const T R0_301 = T(2) * R1_101 + X * R1_201;
    const T R2_110 = X * R3_010;
    const T R1_210 = R2_010 + X * R2_110;
    const T R0_310 = T(2) * R1_110 + X * R1_210;
    const T R3_100 = X * R4_000;
    const T R2_200 = R3_000 + X * R3_100;
    const T R1_300 = T(2) * R2_100 + X * R2_200;
    const T R0_400 = T(3) * R1_200 + X * R1_300;
    const T hp = T(0.5) * invp;
    const T ebx010 = PBx;
    const T ebx011 = hp * (ONE);
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx110 = PAx * ebx010 + ebx011;
    const T ebx111 = hp * (ebx010 + ebx100);
    const T ebx112 = (hp * T(0.5)) * (ebx011 + ebx101);
    const T eby010 = PBy;
    const T eby011 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby110 = PAy * eby010 + eby011;
    const T eby111 = hp * (eby010 + eby100);
    const T eby112 = (hp * T(0.5)) * (eby011 + eby101);
    const T ebz010 = PBz;
    const T ebz011 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz110 = PAz * ebz010 + ebz011;
    const T ebz111 = hp * (ebz010 + ebz100);
    const T ebz112 = (hp * T(0.5)) * (ebz011 + ebz101);
    {
      const T W_000 = fma_t(ekp00_200, R0_200, fma_t(ekp00_100, R0_100, ekp00_000 * R0_000));
      const T W_001 = fma_t(ekp00_200, R0_201, fma_t(ekp00_100, R0_101, ekp00_000 * R0_001));
      const T W_010 = fma_t(ekp00_200, R0_210, fma_t(ekp00_100, R0_110, ekp00_000 * R0_010));
      const T W_100 = fma_t(ekp00_200, R0_300, fma_t(ekp00_100, R0_200, ekp00_000 * R0_100));
      const T W_002 = fma_t(ekp00_200, R0_202, fma_t(ekp00_100, R0_102, ekp00_000 * R0_002));
      const T W_011 = fma_t(ekp00_200, R0_211, fma_t(ekp00_100, R0_111, ekp00_000 * R0_011));
      const T W_020 = fma_t(ekp00_200, R0_220, fma_t(ekp00_100, R0_120, ekp00_000 * R0_020));
      const T W_101 = fma_t(ekp00_200, R0_301, fma_t(ekp00_100, R0_201, ekp00_000 * R0_101));
      const T W_110 = fma_t(ekp00_200, R0_310, fma_t(ekp00_100, R0_210, ekp00_000 * R0_110));
      const T W_200 = fma_t(ekp00_200, R0_400, fma_t(ekp00_100, R0_300, ekp00_000 * R0_200));
      acc[0] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[9] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[18] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[27] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[36] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[45] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[54] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[63] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[72] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp01_110, R0_110, fma_t(ekp01_100, R0_100, fma_t(ekp01_010, R0_010, ekp01_000 * R0_000)));
      const T W_001 = fma_t(ekp01_110, R0_111, fma_t(ekp01_100, R0_101, fma_t(ekp01_010, R0_011, ekp01_000 * R0_001)));
      const T W_010 = fma_t(ekp01_110, R0_120, fma_t(ekp01_100, R0_110, fma_t(ekp01_010, R0_020, ekp01_000 * R0_010)));
      const T W_100 = fma_t(ekp01_110, R0_210, fma_t(ekp01_100, R0_200, fma_t(ekp01_010, R0_110, ekp01_000 * R0_100)));
      const T W_002 = fma_t(ekp01_110, R0_112, fma_t(ekp01_100, R0_102, fma_t(ekp01_010, R0_012, ekp01_000 * R0_002)));
      const T W_011 = fma_t(ekp01_110, R0_121, fma_t(ekp01_100, R0_111, fma_t(ekp01_010, R0_021, ekp01_000 * R0_011)));
      const T W_020 = fma_t(ekp01_110, R0_130, fma_t(ekp01_100, R0_120, fma_t(ekp01_010, R0_030, ekp01_000 * R0_020)));
      const T W_101 = fma_t(ekp01_110, R0_211, fma_t(ekp01_100, R0_201, fma_t(ekp01_010, R0_111, ekp01_000 * R0_101)));
      const T W_110 = fma_t(ekp01_110, R0_220, fma_t(ekp01_100, R0_210, fma_t(ekp01_010, R0_120, ekp01_000 * R0_110)));
      const T W_200 = fma_t(ekp01_110, R0_310, fma_t(ekp01_100, R0_300, fma_t(ekp01_010, R0_210, ekp01_000 * R0_200)));
      acc[1] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[10] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[19] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[28] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[37] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[46] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[55] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[64] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[73] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp02_101, R0_101, fma_t(ekp02_100, R0_100, fma_t(ekp02_001, R0_001, ekp02_000 * R0_000)));
      const T W_001 = fma_t(ekp02_101, R0_102, fma_t(ekp02_100, R0_101, fma_t(ekp02_001, R0_002, ekp02_000 * R0_001)));
      const T W_010 = fma_t(ekp02_101, R0_111, fma_t(ekp02_100, R0_110, fma_t(ekp02_001, R0_011, ekp02_000 * R0_010)));
      const T W_100 = fma_t(ekp02_101, R0_201, fma_t(ekp02_100, R0_200, fma_t(ekp02_001, R0_101, ekp02_000 * R0_100)));
      const T W_002 = fma_t(ekp02_101, R0_103, fma_t(ekp02_100, R0_102, fma_t(ekp02_001, R0_003, ekp02_000 * R0_002)));
      const T W_011 = fma_t(ekp02_101, R0_112, fma_t(ekp02_100, R0_111, fma_t(ekp02_001, R0_012, ekp02_000 * R0_011)));
      const T W_020 = fma_t(ekp02_101, R0_121, fma_t(ekp02_100, R0_120, fma_t(ekp02_001, R0_021, ekp02_000 * R0_020)));
      const T W_101 = fma_t(ekp02_101, R0_202, fma_t(ekp02_100, R0_201, fma_t(ekp02_001, R0_102, ekp02_000 * R0_101)));
      const T W_110 = fma_t(ekp02_101, R0_211, fma_t(ekp02_100, R0_210, fma_t(ekp02_001, R0_111, ekp02_000 * R0_110)));
      const T W_200 = fma_t(ekp02_101, R0_301, fma_t(ekp02_100, R0_300, fma_t(ekp02_001, R0_201, ekp02_000 * R0_200)));
      acc[2] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[11] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[20] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[29] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[38] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[47] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[56] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[65] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[74] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp10_110, R0_110, fma_t(ekp10_100, R0_100, fma_t(ekp10_010, R0_010, ekp10_000 * R0_000)));
      const T W_001 = fma_t(ekp10_110, R0_111, fma_t(ekp10_100, R0_101, fma_t(ekp10_010, R0_011, ekp10_000 * R0_001)));
      const T W_010 = fma_t(ekp10_110, R0_120, fma_t(ekp10_100, R0_110, fma_t(ekp10_010, R0_020, ekp10_000 * R0_010)));
      const T W_100 = fma_t(ekp10_110, R0_210, fma_t(ekp10_100, R0_200, fma_t(ekp10_010, R0_110, ekp10_000 * R0_100)));
      const T W_002 = fma_t(ekp10_110, R0_112, fma_t(ekp10_100, R0_102, fma_t(ekp10_010, R0_012, ekp10_000 * R0_002)));
      const T W_011 = fma_t(ekp10_110, R0_121, fma_t(ekp10_100, R0_111, fma_t(ekp10_010, R0_021, ekp10_000 * R0_011)));
      const T W_020 = fma_t(ekp10_110, R0_130, fma_t(ekp10_100, R0_120, fma_t(ekp10_010, R0_030, ekp10_000 * R0_020)));
      const T W_101 = fma_t(ekp10_110, R0_211, fma_t(ekp10_100, R0_201, fma_t(ekp10_010, R0_111, ekp10_000 * R0_101)));
      const T W_110 = fma_t(ekp10_110, R0_220, fma_t(ekp10_100, R0_210, fma_t(ekp10_010, R0_120, ekp10_000 * R0_110)));
      const T W_200 = fma_t(ekp10_110, R0_310, fma_t(ekp10_100, R0_300, fma_t(ekp10_010, R0_210, ekp10_000 * R0_200)));
      acc[3] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[12] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[21] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[30] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[39] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[48] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[57] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[66] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[75] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp11_020, R0_020, fma_t(ekp11_010, R0_010, ekp11_000 * R0_000));
      const T W_001 = fma_t(ekp11_020, R0_021, fma_t(ekp11_010, R0_011, ekp11_000 * R0_001));
      const T W_010 = fma_t(ekp11_020, R0_030, fma_t(ekp11_010, R0_020, ekp11_000 * R0_010));
      const T W_100 = fma_t(ekp11_020, R0_120, fma_t(ekp11_010, R0_110, ekp11_000 * R0_100));
      const T W_002 = fma_t(ekp11_020, R0_022, fma_t(ekp11_010, R0_012, ekp11_000 * R0_002));
      const T W_011 = fma_t(ekp11_020, R0_031, fma_t(ekp11_010, R0_021, ekp11_000 * R0_011));
      const T W_020 = fma_t(ekp11_020, R0_040, fma_t(ekp11_010, R0_030, ekp11_000 * R0_020));
      const T W_101 = fma_t(ekp11_020, R0_121, fma_t(ekp11_010, R0_111, ekp11_000 * R0_101));
      const T W_110 = fma_t(ekp11_020, R0_130, fma_t(ekp11_010, R0_120, ekp11_000 * R0_110));
      const T W_200 = fma_t(ekp11_020, R0_220, fma_t(ekp11_010, R0_210, ekp11_000 * R0_200));
      acc[4] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[13] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[22] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[31] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[40] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[49] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[58] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[67] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[76] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp12_011, R0_011, fma_t(ekp12_010, R0_010, fma_t(ekp12_001, R0_001, ekp12_000 * R0_000)));
      const T W_001 = fma_t(ekp12_011, R0_012, fma_t(ekp12_010, R0_011, fma_t(ekp12_001, R0_002, ekp12_000 * R0_001)));
      const T W_010 = fma_t(ekp12_011, R0_021, fma_t(ekp12_010, R0_020, fma_t(ekp12_001, R0_011, ekp12_000 * R0_010)));
      const T W_100 = fma_t(ekp12_011, R0_111, fma_t(ekp12_010, R0_110, fma_t(ekp12_001, R0_101, ekp12_000 * R0_100)));
      const T W_002 = fma_t(ekp12_011, R0_013, fma_t(ekp12_010, R0_012, fma_t(ekp12_001, R0_003, ekp12_000 * R0_002)));
      const T W_011 = fma_t(ekp12_011, R0_022, fma_t(ekp12_010, R0_021, fma_t(ekp12_001, R0_012, ekp12_000 * R0_011)));
      const T W_020 = fma_t(ekp12_011, R0_031, fma_t(ekp12_010, R0_030, fma_t(ekp12_001, R0_021, ekp12_000 * R0_020)));
      const T W_101 = fma_t(ekp12_011, R0_112, fma_t(ekp12_010, R0_111, fma_t(ekp12_001, R0_102, ekp12_000 * R0_101)));
      const T W_110 = fma_t(ekp12_011, R0_121, fma_t(ekp12_010, R0_120, fma_t(ekp12_001, R0_111, ekp12_000 * R0_110)));
      const T W_200 = fma_t(ekp12_011, R0_211, fma_t(ekp12_010, R0_210, fma_t(ekp12_001, R0_201, ekp12_000 * R0_200)));
      acc[5] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[14] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[23] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[32] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[41] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[50] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[59] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[68] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[77] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp20_101, R0_101, fma_t(ekp20_100, R0_100, fma_t(ekp20_001, R0_001, ekp20_000 * R0_000)));
      const T W_001 = fma_t(ekp20_101, R0_102, fma_t(ekp20_100, R0_101, fma_t(ekp20_001, R0_002, ekp20_000 * R0_001)));
      const T W_010 = fma_t(ekp20_101, R0_111, fma_t(ekp20_100, R0_110, fma_t(ekp20_001, R0_011, ekp20_000 * R0_010)));
      const T W_100 = fma_t(ekp20_101, R0_201, fma_t(ekp20_100, R0_200, fma_t(ekp20_001, R0_101, ekp20_000 * R0_100)));
      const T W_002 = fma_t(ekp20_101, R0_103, fma_t(ekp20_100, R0_102, fma_t(ekp20_001, R0_003, ekp20_000 * R0_002)));
      const T W_011 = fma_t(ekp20_101, R0_112, fma_t(ekp20_100, R0_111, fma_t(ekp20_001, R0_012, ekp20_000 * R0_011)));
      const T W_020 = fma_t(ekp20_101, R0_121, fma_t(ekp20_100, R0_120, fma_t(ekp20_001, R0_021, ekp20_000 * R0_020)));
      const T W_101 = fma_t(ekp20_101, R0_202, fma_t(ekp20_100, R0_201, fma_t(ekp20_001, R0_102, ekp20_000 * R0_101)));
      const T W_110 = fma_t(ekp20_101, R0_211, fma_t(ekp20_100, R0_210, fma_t(ekp20_001, R0_111, ekp20_000 * R0_110)));
      const T W_200 = fma_t(ekp20_101, R0_301, fma_t(ekp20_100, R0_300, fma_t(ekp20_001, R0_201, ekp20_000 * R0_200)));
      acc[6] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[15] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[24] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[33] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[42] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[51] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[60] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[69] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[78] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp21_011, R0_011, fma_t(ekp21_010, R0_010, fma_t(ekp21_001, R0_001, ekp21_000 * R0_000)));
      const T W_001 = fma_t(ekp21_011, R0_012, fma_t(ekp21_010, R0_011, fma_t(ekp21_001, R0_002, ekp21_000 * R0_001)));
      const T W_010 = fma_t(ekp21_011, R0_021, fma_t(ekp21_010, R0_020, fma_t(ekp21_001, R0_011, ekp21_000 * R0_010)));
      const T W_100 = fma_t(ekp21_011, R0_111, fma_t(ekp21_010, R0_110, fma_t(ekp21_001, R0_101, ekp21_000 * R0_100)));
      const T W_002 = fma_t(ekp21_011, R0_013, fma_t(ekp21_010, R0_012, fma_t(ekp21_001, R0_003, ekp21_000 * R0_002)));
      const T W_011 = fma_t(ekp21_011, R0_022, fma_t(ekp21_010, R0_021, fma_t(ekp21_001, R0_012, ekp21_000 * R0_011)));
      const T W_020 = fma_t(ekp21_011, R0_031, fma_t(ekp21_010, R0_030, fma_t(ekp21_001, R0_021, ekp21_000 * R0_020)));
      const T W_101 = fma_t(ekp21_011, R0_112, fma_t(ekp21_010, R0_111, fma_t(ekp21_001, R0_102, ekp21_000 * R0_101)));
      const T W_110 = fma_t(ekp21_011, R0_121, fma_t(ekp21_010, R0_120, fma_t(ekp21_001, R0_111, ekp21_000 * R0_110)));
      const T W_200 = fma_t(ekp21_011, R0_211, fma_t(ekp21_010, R0_210, fma_t(ekp21_001, R0_201, ekp21_000 * R0_200)));
      acc[7] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[16] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[25] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[34] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[43] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[52] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[61] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[70] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[79] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
    {
      const T W_000 = fma_t(ekp22_002, R0_002, fma_t(ekp22_001, R0_001, ekp22_000 * R0_000));
      const T W_001 = fma_t(ekp22_002, R0_003, fma_t(ekp22_001, R0_002, ekp22_000 * R0_001));
      const T W_010 = fma_t(ekp22_002, R0_012, fma_t(ekp22_001, R0_011, ekp22_000 * R0_010));
      const T W_100 = fma_t(ekp22_002, R0_102, fma_t(ekp22_001, R0_101, ekp22_000 * R0_100));
      const T W_002 = fma_t(ekp22_002, R0_004, fma_t(ekp22_001, R0_003, ekp22_000 * R0_002));
      const T W_011 = fma_t(ekp22_002, R0_013, fma_t(ekp22_001, R0_012, ekp22_000 * R0_011));
      const T W_020 = fma_t(ekp22_002, R0_022, fma_t(ekp22_001, R0_021, ekp22_000 * R0_020));
      const T W_101 = fma_t(ekp22_002, R0_103, fma_t(ekp22_001, R0_102, ekp22_000 * R0_101));
      const T W_110 = fma_t(ekp22_002, R0_112, fma_t(ekp22_001, R0_111, ekp22_000 * R0_110));
      const T W_200 = fma_t(ekp22_002, R0_202, fma_t(ekp22_001, R0_201, ekp22_000 * R0_200));
      acc[8] += fma_t(ebx112, W_200, fma_t(ebx111, W_100, ebx110 * W_000));
      acc[17] += fma_t(ebx101 * eby011, W_110, fma_t(ebx101 * eby010, W_100, fma_t(ebx100 * eby011, W_010, ebx100 * eby010 * W_000)));
      acc[26] += fma_t(ebx101 * ebz011, W_101, fma_t(ebx101 * ebz010, W_100, fma_t(ebx100 * ebz011, W_001, ebx100 * ebz010 * W_000)));
      acc[35] += fma_t(ebx011 * eby101, W_110, fma_t(ebx011 * eby100, W_100, fma_t(ebx010 * eby101, W_010, ebx010 * eby100 * W_000)));
      acc[44] += fma_t(eby112, W_020, fma_t(eby111, W_010, eby110 * W_000));
      acc[53] += fma_t(eby101 * ebz011, W_011, fma_t(eby101 * ebz010, W_010, fma_t(eby100 * ebz011, W_001, eby100 * ebz010 * W_000)));
      acc[62] += fma_t(ebx011 * ebz101, W_101, fma_t(ebx011 * ebz100, W_100, fma_t(ebx010 * ebz101, W_001, ebx010 * ebz100 * W_000)));
      acc[71] += fma_t(eby011 * ebz101, W_011, fma_t(eby011 * ebz100, W_010, fma_t(eby010 * ebz101, W_001, eby010 * ebz100 * W_000)));
      acc[80] += fma_t(ebz112, W_002, fma_t(ebz111, W_001, ebz110 * W_000));
    }
  }
}

// ---- class (ds|ss): 6x1 integrals, L = 2
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_dsss(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekp00_000 = ONE;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[3];
    boys_eval<T, 2>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T hp = T(0.5) * invp;
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    {
      const T W_000 = ekp00_000 * R0_000;
      const T W_001 = ekp00_000 * R0_001;
      const T W_010 = ekp00_000 * R0_010;
      const T W_100 = ekp00_000 * R0_100;
      const T W_002 = ekp00_000 * R0_002;
      const T W_011 = ekp00_000 * R0_011;
      const T W_020 = ekp00_000 * R0_020;
      const T W_101 = ekp00_000 * R0_101;
      const T W_110 = ekp00_000 * R0_110;
      const T W_200 = ekp00_000 * R0_200;
      acc[0] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[1] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[2] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[3] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[4] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[5] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
  }
}

// ---- class (ds|ps): 6x3 integrals, L = 3
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_dsps(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekp00_000 = ekx100;
  const T ekp00_100 = -(ekx101);
  const T ekp10_000 = eky100;
  const T ekp10_010 = -(eky101);
  const T ekp20_000 = ekz100;
  const T ekp20_001 = -(ekz101);
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[4];
    boys_eval<T, 3>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T hp = T(0.5) * invp;
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    {
      const T W_000 = fma_t(ekp00_100, R0_100, ekp00_000 * R0_000);
      const T W_001 = fma_t(ekp00_100, R0_101, ekp00_000 * R0_001);
      const T W_010 = fma_t(ekp00_100, R0_110, ekp00_000 * R0_010);
      const T W_100 = fma_t(ekp00_100, R0_200, ekp00_000 * R0_100);
      const T W_002 = fma_t(ekp00_100, R0_102, ekp00_000 * R0_002);
      const T W_011 = fma_t(ekp00_100, R0_111, ekp00_000 * R0_011);
      const T W_020 = fma_t(ekp00_100, R0_120, ekp00_000 * R0_020);
      const T W_101 = fma_t(ekp00_100, R0_201, ekp00_000 * R0_101);
      const T W_110 = fma_t(ekp00_100, R0_210, ekp00_000 * R0_110);
      const T W_200 = fma_t(ekp00_100, R0_300, ekp00_000 * R0_200);
      acc[0] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[3] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[6] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[9] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[12] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[15] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp10_010, R0_010, ekp10_000 * R0_000);
      const T W_001 = fma_t(ekp10_010, R0_011, ekp10_000 * R0_001);
      const T W_010 = fma_t(ekp10_010, R0_020, ekp10_000 * R0_010);
      const T W_100 = fma_t(ekp10_010, R0_110, ekp10_000 * R0_100);
      const T W_002 = fma_t(ekp10_010, R0_012, ekp10_000 * R0_002);
      const T W_011 = fma_t(ekp10_010, R0_021, ekp10_000 * R0_011);
      const T W_020 = fma_t(ekp10_010, R0_030, ekp10_000 * R0_020);
      const T W_101 = fma_t(ekp10_010, R0_111, ekp10_000 * R0_101);
      const T W_110 = fma_t(ekp10_010, R0_120, ekp10_000 * R0_110);
      const T W_200 = fma_t(ekp10_010, R0_210, ekp10_000 * R0_200);
      acc[1] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[4] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[7] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[10] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[13] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[16] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp20_001, R0_001, ekp20_000 * R0_000);
      const T W_001 = fma_t(ekp20_001, R0_002, ekp20_000 * R0_001);
      const T W_010 = fma_t(ekp20_001, R0_011, ekp20_000 * R0_010);
      const T W_100 = fma_t(ekp20_001, R0_101, ekp20_000 * R0_100);
      const T W_002 = fma_t(ekp20_001, R0_003, ekp20_000 * R0_002);
      const T W_011 = fma_t(ekp20_001, R0_012, ekp20_000 * R0_011);
      const T W_020 = fma_t(ekp20_001, R0_021, ekp20_000 * R0_020);
      const T W_101 = fma_t(ekp20_001, R0_102, ekp20_000 * R0_101);
      const T W_110 = fma_t(ekp20_001, R0_111, ekp20_000 * R0_110);
      const T W_200 = fma_t(ekp20_001, R0_201, ekp20_000 * R0_200);
      acc[2] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[5] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[8] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[11] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[14] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[17] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
  }
}

// ---- class (ds|pp): 6x9 integrals, L = 4
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_dspp(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx010 = QDx;
  const T ekx011 = hq * (ONE);
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T ekx110 = QCx * ekx010 + ekx011;
  const T ekx111 = hq * (ekx010 + ekx100);
  const T ekx112 = (hq * T(0.5)) * (ekx011 + ekx101);
  const T eky010 = QDy;
  const T eky011 = hq * (ONE);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T eky110 = QCy * eky010 + eky011;
  const T eky111 = hq * (eky010 + eky100);
  const T eky112 = (hq * T(0.5)) * (eky011 + eky101);
  const T ekz010 = QDz;
  const T ekz011 = hq * (ONE);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekz110 = QCz * ekz010 + ekz011;
  const T ekz111 = hq * (ekz010 + ekz100);
  const T ekz112 = (hq * T(0.5)) * (ekz011 + ekz101);
  const T ekp00_000 = ekx110;
  const T ekp00_100 = -(ekx111);
  const T ekp00_200 = ekx112;
  const T ekp01_000 = ekx100 * eky010;
  const T ekp01_010 = -(ekx100 * eky011);
  const T ekp01_100 = -(ekx101 * eky010);
  const T ekp01_110 = ekx101 * eky011;
  const T ekp02_000 = ekx100 * ekz010;
  const T ekp02_001 = -(ekx100 * ekz011);
  const T ekp02_100 = -(ekx101 * ekz010);
  const T ekp02_101 = ekx101 * ekz011;
  const T ekp10_000 = ekx010 * eky100;
  const T ekp10_010 = -(ekx010 * eky101);
  const T ekp10_100 = -(ekx011 * eky100);
  const T ekp10_110 = ekx011 * eky101;
  const T ekp11_000 = eky110;
  const T ekp11_010 = -(eky111);
  const T ekp11_020 = eky112;
  const T ekp12_000 = eky100 * ekz010;
  const T ekp12_001 = -(eky100 * ekz011);
  const T ekp12_010 = -(eky101 * ekz010);
  const T ekp12_011 = eky101 * ekz011;
  const T ekp20_000 = ekx010 * ekz100;
  const T ekp20_001 = -(ekx010 * ekz101);
  const T ekp20_100 = -(ekx011 * ekz100);
  const T ekp20_101 = ekx011 * ekz101;
  const T ekp21_000 = eky010 * ekz100;
  const T ekp21_001 = -(eky010 * ekz101);
  const T ekp21_010 = -(eky011 * ekz100);
  const T ekp21_011 = eky011 * ekz101;
  const T ekp22_000 = ekz110;
  const T ekp22_001 = -(ekz111);
  const T ekp22_002 = ekz112;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[5];
    boys_eval<T, 4>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    scale *= m2a;
    const T R4_000 = scale * F[4];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T R3_001 = Z * R4_000;
    const T R2_002 = R3_000 + Z * R3_001;
    const T R1_003 = T(2) * R2_001 + Z * R2_002;
    const T R0_004 = T(3) * R1_002 + Z * R1_003;
    const T R0_013 = Y * R1_003;
    const T R1_012 = Y * R2_002;
    const T R0_022 = R1_002 + Y * R1_012;
    const T R2_011 = Y * R3_001;
    const T R1_021 = R2_001 + Y * R2_011;
    const T R0_031 = T(2) * R1_011 + Y * R1_021;
    const T R3_010 = Y * R4_000;
    const T R2_020 = R3_000 + Y * R3_010;
    const T R1_030 = T(2) * R2_010 + Y * R2_020;
    const T R0_040 = T(3) * R1_020 + Y * R1_030;
    const T R0_103 = X * R1_003;
    const T R0_112 = X * R1_012;
    const T R0_121 = X * R1_021;
    const T R0_130 = X * R1_030;
    const T R1_102 = X * R2_002;
    const T R0_202 = R1_002 + X * R1_102;
    const T R1_111 = X * R2_011;
    const T R0_211 = R1_011 + X * R1_111;
    const T R1_120 = X * R2_020;
    const T R0_220 = R1_020 + X * R1_120;
    const T R2_101 = X * R3_001;
    const T R1_201 = R2_001 + X * R2_101;
    const T R0_301 = T(2) * R1_101 + X * R1_201;
    const T R2_110 = X * R3_010;
    const T R1_210 = R2_010 + X * R2_110;
    const T R0_310 = T(2) * R1_110 + X * R1_210;
    const T R3_100 = X * R4_000;
    const T R2_200 = R3_000 + X * R3_100;
    const T R1_300 = T(2) * R2_100 + X * R2_200;
    const T R0_400 = T(3) * R1_200 + X * R1_300;
    const T hp = T(0.5) * invp;
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    {
      const T W_000 = fma_t(ekp00_200, R0_200, fma_t(ekp00_100, R0_100, ekp00_000 * R0_000));
      const T W_001 = fma_t(ekp00_200, R0_201, fma_t(ekp00_100, R0_101, ekp00_000 * R0_001));
      const T W_010 = fma_t(ekp00_200, R0_210, fma_t(ekp00_100, R0_110, ekp00_000 * R0_010));
      const T W_100 = fma_t(ekp00_200, R0_300, fma_t(ekp00_100, R0_200, ekp00_000 * R0_100));
      const T W_002 = fma_t(ekp00_200, R0_202, fma_t(ekp00_100, R0_102, ekp00_000 * R0_002));
      const T W_011 = fma_t(ekp00_200, R0_211, fma_t(ekp00_100, R0_111, ekp00_000 * R0_011));
      const T W_020 = fma_t(ekp00_200, R0_220, fma_t(ekp00_100, R0_120, ekp00_000 * R0_020));
      const T W_101 = fma_t(ekp00_200, R0_301, fma_t(ekp00_100, R0_201, ekp00_000 * R0_101));
      const T W_110 = fma_t(ekp00_200, R0_310, fma_t(ekp00_100, R0_210, ekp00_000 * R0_110));
      const T W_200 = fma_t(ekp00_200, R0_400, fma_t(ekp00_100, R0_300, ekp00_000 * R0_200));
      acc[0] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[9] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[18] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[27] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[36] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[45] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp01_110, R0_110, fma_t(ekp01_100, R0_100, fma_t(ekp01_010, R0_010, ekp01_000 * R0_000)));
      const T W_001 = fma_t(ekp01_110, R0_111, fma_t(ekp01_100, R0_101, fma_t(ekp01_010, R0_011, ekp01_000 * R0_001)));
      const T W_010 = fma_t(ekp01_110, R0_120, fma_t(ekp01_100, R0_110, fma_t(ekp01_010, R0_020, ekp01_000 * R0_010)));
      const T W_100 = fma_t(ekp01_110, R0_210, fma_t(ekp01_100, R0_200, fma_t(ekp01_010, R0_110, ekp01_000 * R0_100)));
      const T W_002 = fma_t(ekp01_110, R0_112, fma_t(ekp01_100, R0_102, fma_t(ekp01_010, R0_012, ekp01_000 * R0_002)));
      const T W_011 = fma_t(ekp01_110, R0_121, fma_t(ekp01_100, R0_111, fma_t(ekp01_010, R0_021, ekp01_000 * R0_011)));
      const T W_020 = fma_t(ekp01_110, R0_130, fma_t(ekp01_100, R0_120, fma_t(ekp01_010, R0_030, ekp01_000 * R0_020)));
      const T W_101 = fma_t(ekp01_110, R0_211, fma_t(ekp01_100, R0_201, fma_t(ekp01_010, R0_111, ekp01_000 * R0_101)));
      const T W_110 = fma_t(ekp01_110, R0_220, fma_t(ekp01_100, R0_210, fma_t(ekp01_010, R0_120, ekp01_000 * R0_110)));
      const T W_200 = fma_t(ekp01_110, R0_310, fma_t(ekp01_100, R0_300, fma_t(ekp01_010, R0_210, ekp01_000 * R0_200)));
      acc[1] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[10] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[19] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[28] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[37] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[46] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp02_101, R0_101, fma_t(ekp02_100, R0_100, fma_t(ekp02_001, R0_001, ekp02_000 * R0_000)));
      const T W_001 = fma_t(ekp02_101, R0_102, fma_t(ekp02_100, R0_101, fma_t(ekp02_001, R0_002, ekp02_000 * R0_001)));
      const T W_010 = fma_t(ekp02_101, R0_111, fma_t(ekp02_100, R0_110, fma_t(ekp02_001, R0_011, ekp02_000 * R0_010)));
      const T W_100 = fma_t(ekp02_101, R0_201, fma_t(ekp02_100, R0_200, fma_t(ekp02_001, R0_101, ekp02_000 * R0_100)));
      const T W_002 = fma_t(ekp02_101, R0_103, fma_t(ekp02_100, R0_102, fma_t(ekp02_001, R0_003, ekp02_000 * R0_002)));
      const T W_011 = fma_t(ekp02_101, R0_112, fma_t(ekp02_100, R0_111, fma_t(ekp02_001, R0_012, ekp02_000 * R0_011)));
      const T W_020 = fma_t(ekp02_101, R0_121, fma_t(ekp02_100, R0_120, fma_t(ekp02_001, R0_021, ekp02_000 * R0_020)));
      const T W_101 = fma_t(ekp02_101, R0_202, fma_t(ekp02_100, R0_201, fma_t(ekp02_001, R0_102, ekp02_000 * R0_101)));
      const T W_110 = fma_t(ekp02_101, R0_211, fma_t(ekp02_100, R0_210, fma_t(ekp02_001, R0_111, ekp02_000 * R0_110)));
      const T W_200 = fma_t(ekp02_101, R0_301, fma_t(ekp02_100, R0_300, fma_t(ekp02_001, R0_201, ekp02_000 * R0_200)));
      acc[2] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[11] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[20] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[29] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[38] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[47] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp10_110, R0_110, fma_t(ekp10_100, R0_100, fma_t(ekp10_010, R0_010, ekp10_000 * R0_000)));
      const T W_001 = fma_t(ekp10_110, R0_111, fma_t(ekp10_100, R0_101, fma_t(ekp10_010, R0_011, ekp10_000 * R0_001)));
      const T W_010 = fma_t(ekp10_110, R0_120, fma_t(ekp10_100, R0_110, fma_t(ekp10_010, R0_020, ekp10_000 * R0_010)));
      const T W_100 = fma_t(ekp10_110, R0_210, fma_t(ekp10_100, R0_200, fma_t(ekp10_010, R0_110, ekp10_000 * R0_100)));
      const T W_002 = fma_t(ekp10_110, R0_112, fma_t(ekp10_100, R0_102, fma_t(ekp10_010, R0_012, ekp10_000 * R0_002)));
      const T W_011 = fma_t(ekp10_110, R0_121, fma_t(ekp10_100, R0_111, fma_t(ekp10_010, R0_021, ekp10_000 * R0_011)));
      const T W_020 = fma_t(ekp10_110, R0_130, fma_t(ekp10_100, R0_120, fma_t(ekp10_010, R0_030, ekp10_000 * R0_020)));
      const T W_101 = fma_t(ekp10_110, R0_211, fma_t(ekp10_100, R0_201, fma_t(ekp10_010, R0_111, ekp10_000 * R0_101)));
      const T W_110 = fma_t(ekp10_110, R0_220, fma_t(ekp10_100, R0_210, fma_t(ekp10_010, R0_120, ekp10_000 * R0_110)));
      const T W_200 = fma_t(ekp10_110, R0_310, fma_t(ekp10_100, R0_300, fma_t(ekp10_010, R0_210, ekp10_000 * R0_200)));
      acc[3] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[12] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[21] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[30] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[39] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[48] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp11_020, R0_020, fma_t(ekp11_010, R0_010, ekp11_000 * R0_000));
      const T W_001 = fma_t(ekp11_020, R0_021, fma_t(ekp11_010, R0_011, ekp11_000 * R0_001));
      const T W_010 = fma_t(ekp11_020, R0_030, fma_t(ekp11_010, R0_020, ekp11_000 * R0_010));
      const T W_100 = fma_t(ekp11_020, R0_120, fma_t(ekp11_010, R0_110, ekp11_000 * R0_100));
      const T W_002 = fma_t(ekp11_020, R0_022, fma_t(ekp11_010, R0_012, ekp11_000 * R0_002));
      const T W_011 = fma_t(ekp11_020, R0_031, fma_t(ekp11_010, R0_021, ekp11_000 * R0_011));
      const T W_020 = fma_t(ekp11_020, R0_040, fma_t(ekp11_010, R0_030, ekp11_000 * R0_020));
      const T W_101 = fma_t(ekp11_020, R0_121, fma_t(ekp11_010, R0_111, ekp11_000 * R0_101));
      const T W_110 = fma_t(ekp11_020, R0_130, fma_t(ekp11_010, R0_120, ekp11_000 * R0_110));
      const T W_200 = fma_t(ekp11_020, R0_220, fma_t(ekp11_010, R0_210, ekp11_000 * R0_200));
      acc[4] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[13] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[22] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[31] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[40] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[49] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp12_011, R0_011, fma_t(ekp12_010, R0_010, fma_t(ekp12_001, R0_001, ekp12_000 * R0_000)));
      const T W_001 = fma_t(ekp12_011, R0_012, fma_t(ekp12_010, R0_011, fma_t(ekp12_001, R0_002, ekp12_000 * R0_001)));
      const T W_010 = fma_t(ekp12_011, R0_021, fma_t(ekp12_010, R0_020, fma_t(ekp12_001, R0_011, ekp12_000 * R0_010)));
      const T W_100 = fma_t(ekp12_011, R0_111, fma_t(ekp12_010, R0_110, fma_t(ekp12_001, R0_101, ekp12_000 * R0_100)));
      const T W_002 = fma_t(ekp12_011, R0_013, fma_t(ekp12_010, R0_012, fma_t(ekp12_001, R0_003, ekp12_000 * R0_002)));
      const T W_011 = fma_t(ekp12_011, R0_022, fma_t(ekp12_010, R0_021, fma_t(ekp12_001, R0_012, ekp12_000 * R0_011)));
      const T W_020 = fma_t(ekp12_011, R0_031, fma_t(ekp12_010, R0_030, fma_t(ekp12_001, R0_021, ekp12_000 * R0_020)));
      const T W_101 = fma_t(ekp12_011, R0_112, fma_t(ekp12_010, R0_111, fma_t(ekp12_001, R0_102, ekp12_000 * R0_101)));
      const T W_110 = fma_t(ekp12_011, R0_121, fma_t(ekp12_010, R0_120, fma_t(ekp12_001, R0_111, ekp12_000 * R0_110)));
      const T W_200 = fma_t(ekp12_011, R0_211, fma_t(ekp12_010, R0_210, fma_t(ekp12_001, R0_201, ekp12_000 * R0_200)));
      acc[5] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[14] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[23] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[32] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[41] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[50] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp20_101, R0_101, fma_t(ekp20_100, R0_100, fma_t(ekp20_001, R0_001, ekp20_000 * R0_000)));
      const T W_001 = fma_t(ekp20_101, R0_102, fma_t(ekp20_100, R0_101, fma_t(ekp20_001, R0_002, ekp20_000 * R0_001)));
      const T W_010 = fma_t(ekp20_101, R0_111, fma_t(ekp20_100, R0_110, fma_t(ekp20_001, R0_011, ekp20_000 * R0_010)));
      const T W_100 = fma_t(ekp20_101, R0_201, fma_t(ekp20_100, R0_200, fma_t(ekp20_001, R0_101, ekp20_000 * R0_100)));
      const T W_002 = fma_t(ekp20_101, R0_103, fma_t(ekp20_100, R0_102, fma_t(ekp20_001, R0_003, ekp20_000 * R0_002)));
      const T W_011 = fma_t(ekp20_101, R0_112, fma_t(ekp20_100, R0_111, fma_t(ekp20_001, R0_012, ekp20_000 * R0_011)));
      const T W_020 = fma_t(ekp20_101, R0_121, fma_t(ekp20_100, R0_120, fma_t(ekp20_001, R0_021, ekp20_000 * R0_020)));
      const T W_101 = fma_t(ekp20_101, R0_202, fma_t(ekp20_100, R0_201, fma_t(ekp20_001, R0_102, ekp20_000 * R0_101)));
      const T W_110 = fma_t(ekp20_101, R0_211, fma_t(ekp20_100, R0_210, fma_t(ekp20_001, R0_111, ekp20_000 * R0_110)));
      const T W_200 = fma_t(ekp20_101, R0_301, fma_t(ekp20_100, R0_300, fma_t(ekp20_001, R0_201, ekp20_000 * R0_200)));
      acc[6] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[15] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[24] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[33] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[42] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[51] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp21_011, R0_011, fma_t(ekp21_010, R0_010, fma_t(ekp21_001, R0_001, ekp21_000 * R0_000)));
      const T W_001 = fma_t(ekp21_011, R0_012, fma_t(ekp21_010, R0_011, fma_t(ekp21_001, R0_002, ekp21_000 * R0_001)));
      const T W_010 = fma_t(ekp21_011, R0_021, fma_t(ekp21_010, R0_020, fma_t(ekp21_001, R0_011, ekp21_000 * R0_010)));
      const T W_100 = fma_t(ekp21_011, R0_111, fma_t(ekp21_010, R0_110, fma_t(ekp21_001, R0_101, ekp21_000 * R0_100)));
      const T W_002 = fma_t(ekp21_011, R0_013, fma_t(ekp21_010, R0_012, fma_t(ekp21_001, R0_003, ekp21_000 * R0_002)));
      const T W_011 = fma_t(ekp21_011, R0_022, fma_t(ekp21_010, R0_021, fma_t(ekp21_001, R0_012, ekp21_000 * R0_011)));
      const T W_020 = fma_t(ekp21_011, R0_031, fma_t(ekp21_010, R0_030, fma_t(ekp21_001, R0_021, ekp21_000 * R0_020)));
      const T W_101 = fma_t(ekp21_011, R0_112, fma_t(ekp21_010, R0_111, fma_t(ekp21_001, R0_102, ekp21_000 * R0_101)));
      const T W_110 = fma_t(ekp21_011, R0_121, fma_t(ekp21_010, R0_120, fma_t(ekp21_001, R0_111, ekp21_000 * R0_110)));
      const T W_200 = fma_t(ekp21_011, R0_211, fma_t(ekp21_010, R0_210, fma_t(ekp21_001, R0_201, ekp21_000 * R0_200)));
      acc[7] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[16] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[25] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[34] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[43] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[52] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp22_002, R0_002, fma_t(ekp22_001, R0_001, ekp22_000 * R0_000));
      const T W_001 = fma_t(ekp22_002, R0_003, fma_t(ekp22_001, R0_002, ekp22_000 * R0_001));
      const T W_010 = fma_t(ekp22_002, R0_012, fma_t(ekp22_001, R0_011, ekp22_000 * R0_010));
      const T W_100 = fma_t(ekp22_002, R0_102, fma_t(ekp22_001, R0_101, ekp22_000 * R0_100));
      const T W_002 = fma_t(ekp22_002, R0_004, fma_t(ekp22_001, R0_003, ekp22_000 * R0_002));
      const T W_011 = fma_t(ekp22_002, R0_013, fma_t(ekp22_001, R0_012, ekp22_000 * R0_011));
      const T W_020 = fma_t(ekp22_002, R0_022, fma_t(ekp22_001, R0_021, ekp22_000 * R0_020));
      const T W_101 = fma_t(ekp22_002, R0_103, fma_t(ekp22_001, R0_102, ekp22_000 * R0_101));
      const T W_110 = fma_t(ekp22_002, R0_112, fma_t(ekp22_001, R0_111, ekp22_000 * R0_110));
      const T W_200 = fma_t(ekp22_002, R0_202, fma_t(ekp22_001, R0_201, ekp22_000 * R0_200));
      acc[8] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[17] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[26] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[35] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[44] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[53] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
  }
}

// ---- class (ds|ds): 6x6 integrals, L = 4
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_dsds(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T ekx200 = QCx * ekx100 + ekx101;
  const T ekx201 = hq * (T(2) * ekx100);
  const T ekx202 = (hq * T(0.5)) * (T(2) * ekx101);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T eky200 = QCy * eky100 + eky101;
  const T eky201 = hq * (T(2) * eky100);
  const T eky202 = (hq * T(0.5)) * (T(2) * eky101);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekz200 = QCz * ekz100 + ekz101;
  const T ekz201 = hq * (T(2) * ekz100);
  const T ekz202 = (hq * T(0.5)) * (T(2) * ekz101);
  const T ekp00_000 = ekx200;
  const T ekp00_100 = -(ekx201);
  const T ekp00_200 = ekx202;
  const T ekp10_000 = ekx100 * eky100;
  const T ekp10_010 = -(ekx100 * eky101);
  const T ekp10_100 = -(ekx101 * eky100);
  const T ekp10_110 = ekx101 * eky101;
  const T ekp20_000 = ekx100 * ekz100;
  const T ekp20_001 = -(ekx100 * ekz101);
  const T ekp20_100 = -(ekx101 * ekz100);
  const T ekp20_101 = ekx101 * ekz101;
  const T ekp30_000 = eky200;
  const T ekp30_010 = -(eky201);
  const T ekp30_020 = eky202;
  const T ekp40_000 = eky100 * ekz100;
  const T ekp40_001 = -(eky100 * ekz101);
  const T ekp40_010 = -(eky101 * ekz100);
  const T ekp40_011 = eky101 * ekz101;
  const T ekp50_000 = ekz200;
  const T ekp50_001 = -(ekz201);
  const T ekp50_002 = ekz202;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[5];
    boys_eval<T, 4>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    scale *= m2a;
    const T R4_000 = scale * F[4];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T R3_001 = Z * R4_000;
    const T R2_002 = R3_000 + Z * R3_001;
    const T R1_003 = T(2) * R2_001 + Z * R2_002;
    const T R0_004 = T(3) * R1_002 + Z * R1_003;
    const T R0_013 = Y * R1_003;
    const T R1_012 = Y * R2_002;
    const T R0_022 = R1_002 + Y * R1_012;
    const T R2_011 = Y * R3_001;
    const T R1_021 = R2_001 + Y * R2_011;
    const T R0_031 = T(2) * R1_011 + Y * R1_021;
    const T R3_010 = Y * R4_000;
    const T R2_020 = R3_000 + Y * R3_010;
    const T R1_030 = T(2) * R2_010 + Y * R2_020;
    const T R0_040 = T(3) * R1_020 + Y * R1_030;
    const T R0_103 = X * R1_003;
    const T R0_112 = X * R1_012;
    const T R0_121 = X * R1_021;
    const T R0_130 = X * R1_030;
    const T R1_102 = X * R2_002;
    const T R0_202 = R1_002 + X * R1_102;
    const T R1_111 = X * R2_011;
    const T R0_211 = R1_011 + X * R1_111;
    const T R1_120 = X * R2_020;
    const T R0_220 = R1_020 + X * R1_120;
    const T R2_101 = X * R3_001;
    const T R1_201 = R2_001 + X * R2_101;
    const T R0_301 = T(2) * R1_101 + X * R1_201;
    const T R2_110 = X * R3_010;
    const T R1_210 = R2_010 + X * R2_110;
    const T R0_310 = T(2) * R1_110 + X * R1_210;
    const T R3_100 = X * R4_000;
    const T R2_200 = R3_000 + X * R3_100;
    const T R1_300 = T(2) * R2_100 + X * R2_200;
    const T R0_400 = T(3) * R1_200 + X * R1_300;
    const T hp = T(0.5) * invp;
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    {
      const T W_000 = fma_t(ekp00_200, R0_200, fma_t(ekp00_100, R0_100, ekp00_000 * R0_000));
      const T W_001 = fma_t(ekp00_200, R0_201, fma_t(ekp00_100, R0_101, ekp00_000 * R0_001));
      const T W_010 = fma_t(ekp00_200, R0_210, fma_t(ekp00_100, R0_110, ekp00_000 * R0_010));
      const T W_100 = fma_t(ekp00_200, R0_300, fma_t(ekp00_100, R0_200, ekp00_000 * R0_100));
      const T W_002 = fma_t(ekp00_200, R0_202, fma_t(ekp00_100, R0_102, ekp00_000 * R0_002));
      const T W_011 = fma_t(ekp00_200, R0_211, fma_t(ekp00_100, R0_111, ekp00_000 * R0_011));
      const T W_020 = fma_t(ekp00_200, R0_220, fma_t(ekp00_100, R0_120, ekp00_000 * R0_020));
      const T W_101 = fma_t(ekp00_200, R0_301, fma_t(ekp00_100, R0_201, ekp00_000 * R0_101));
      const T W_110 = fma_t(ekp00_200, R0_310, fma_t(ekp00_100, R0_210, ekp00_000 * R0_110));
      const T W_200 = fma_t(ekp00_200, R0_400, fma_t(ekp00_100, R0_300, ekp00_000 * R0_200));
      acc[0] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[6] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[12] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[18] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[24] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[30] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp10_110, R0_110, fma_t(ekp10_100, R0_100, fma_t(ekp10_010, R0_010, ekp10_000 * R0_000)));
      const T W_001 = fma_t(ekp10_110, R0_111, fma_t(ekp10_100, R0_101, fma_t(ekp10_010, R0_011, ekp10_000 * R0_001)));
      const T W_010 = fma_t(ekp10_110, R0_120, fma_t(ekp10_100, R0_110, fma_t(ekp10_010, R0_020, ekp10_000 * R0_010)));
      const T W_100 = fma_t(ekp10_110, R0_210, fma_t(ekp10_100, R0_200, fma_t(ekp10_010, R0_110, ekp10_000 * R0_100)));
      const T W_002 = fma_t(ekp10_110, R0_112, fma_t(ekp10_100, R0_102, fma_t(ekp10_010, R0_012, ekp10_000 * R0_002)));
      const T W_011 = fma_t(ekp10_110, R0_121, fma_t(ekp10_100, R0_111, fma_t(ekp10_010, R0_021, ekp10_000 * R0_011)));
      const T W_020 = fma_t(ekp10_110, R0_130, fma_t(ekp10_100, R0_120, fma_t(ekp10_010, R0_030, ekp10_000 * R0_020)));
      const T W_101 = fma_t(ekp10_110, R0_211, fma_t(ekp10_100, R0_201, fma_t(ekp10_010, R0_111, ekp10_000 * R0_101)));
      const T W_110 = fma_t(ekp10_110, R0_220, fma_t(ekp10_100, R0_210, fma_t(ekp10_010, R0_120, ekp10_000 * R0_110)));
      const T W_200 = fma_t(ekp10_110, R0_310, fma_t(ekp10_100, R0_300, fma_t(ekp10_010, R0_210, ekp10_000 * R0_200)));
      acc[1] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[7] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[13] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[19] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[25] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[31] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp20_101, R0_101, fma_t(ekp20_100, R0_100, fma_t(ekp20_001, R0_001, ekp20_000 * R0_000)));
      const T W_001 = fma_t(ekp20_101, R0_102, fma_t(ekp20_100, R0_101, fma_t(ekp20_001, R0_002, ekp20_000 * R0_001)));
      const T W_010 = fma_t(ekp20_101, R0_111, fma_t(ekp20_100, R0_110, fma_t(ekp20_001, R0_011, ekp20_000 * R0_010)));
      const T W_100 = fma_t(ekp20_101, R0_201, fma_t(ekp20_100, R0_200, fma_t(ekp20_001, R0_101, ekp20_000 * R0_100)));
      const T W_002 = fma_t(ekp20_101, R0_103, fma_t(ekp20_100, R0_102, fma_t(ekp20_001, R0_003, ekp20_000 * R0_002)));
      const T W_011 = fma_t(ekp20_101, R0_112, fma_t(ekp20_100, R0_111, fma_t(ekp20_001, R0_012, ekp20_000 * R0_011)));
      const T W_020 = fma_t(ekp20_101, R0_121, fma_t(ekp20_100, R0_120, fma_t(ekp20_001, R0_021, ekp20_000 * R0_020)));
      const T W_101 = fma_t(ekp20_101, R0_202, fma_t(ekp20_100, R0_201, fma_t(ekp20_001, R0_102, ekp20_000 * R0_101)));
      const T W_110 = fma_t(ekp20_101, R0_211, fma_t(ekp20_100, R0_210, fma_t(ekp20_001, R0_111, ekp20_000 * R0_110)));
      const T W_200 = fma_t(ekp20_101, R0_301, fma_t(ekp20_100, R0_300, fma_t(ekp20_001, R0_201, ekp20_000 * R0_200)));
      acc[2] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[8] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[14] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[20] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[26] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[32] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp30_020, R0_020, fma_t(ekp30_010, R0_010, ekp30_000 * R0_000));
      const T W_001 = fma_t(ekp30_020, R0_021, fma_t(ekp30_010, R0_011, ekp30_000 * R0_001));
      const T W_010 = fma_t(ekp30_020, R0_030, fma_t(ekp30_010, R0_020, ekp30_000 * R0_010));
      const T W_100 = fma_t(ekp30_020, R0_120, fma_t(ekp30_010, R0_110, ekp30_000 * R0_100));
      const T W_002 = fma_t(ekp30_020, R0_022, fma_t(ekp30_010, R0_012, ekp30_000 * R0_002));
      const T W_011 = fma_t(ekp30_020, R0_031, fma_t(ekp30_010, R0_021, ekp30_000 * R0_011));
      const T W_020 = fma_t(ekp30_020, R0_040, fma_t(ekp30_010, R0_030, ekp30_000 * R0_020));
      const T W_101 = fma_t(ekp30_020, R0_121, fma_t(ekp30_010, R0_111, ekp30_000 * R0_101));
      const T W_110 = fma_t(ekp30_020, R0_130, fma_t(ekp30_010, R0_120, ekp30_000 * R0_110));
      const T W_200 = fma_t(ekp30_020, R0_220, fma_t(ekp30_010, R0_210, ekp30_000 * R0_200));
      acc[3] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[9] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[15] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[21] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[27] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[33] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp40_011, R0_011, fma_t(ekp40_010, R0_010, fma_t(ekp40_001, R0_001, ekp40_000 * R0_000)));
      const T W_001 = fma_t(ekp40_011, R0_012, fma_t(ekp40_010, R0_011, fma_t(ekp40_001, R0_002, ekp40_000 * R0_001)));
      const T W_010 = fma_t(ekp40_011, R0_021, fma_t(ekp40_010, R0_020, fma_t(ekp40_001, R0_011, ekp40_000 * R0_010)));
      const T W_100 = fma_t(ekp40_011, R0_111, fma_t(ekp40_010, R0_110, fma_t(ekp40_001, R0_101, ekp40_000 * R0_100)));
      const T W_002 = fma_t(ekp40_011, R0_013, fma_t(ekp40_010, R0_012, fma_t(ekp40_001, R0_003, ekp40_000 * R0_002)));
      const T W_011 = fma_t(ekp40_011, R0_022, fma_t(ekp40_010, R0_021, fma_t(ekp40_001, R0_012, ekp40_000 * R0_011)));
      const T W_020 = fma_t(ekp40_011, R0_031, fma_t(ekp40_010, R0_030, fma_t(ekp40_001, R0_021, ekp40_000 * R0_020)));
      const T W_101 = fma_t(ekp40_011, R0_112, fma_t(ekp40_010, R0_111, fma_t(ekp40_001, R0_102, ekp40_000 * R0_101)));
      const T W_110 = fma_t(ekp40_011, R0_121, fma_t(ekp40_010, R0_120, fma_t(ekp40_001, R0_111, ekp40_000 * R0_110)));
      const T W_200 = fma_t(ekp40_011, R0_211, fma_t(ekp40_010, R0_210, fma_t(ekp40_001, R0_201, ekp40_000 * R0_200)));
      acc[4] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[10] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[16] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[22] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[28] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[34] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
    {
      const T W_000 = fma_t(ekp50_002, R0_002, fma_t(ekp50_001, R0_001, ekp50_000 * R0_000));
      const T W_001 = fma_t(ekp50_002, R0_003, fma_t(ekp50_001, R0_002, ekp50_000 * R0_001));
      const T W_010 = fma_t(ekp50_002, R0_012, fma_t(ekp50_001, R0_011, ekp50_000 * R0_010));
      const T W_100 = fma_t(ekp50_002, R0_102, fma_t(ekp50_001, R0_101, ekp50_000 * R0_100));
      const T W_002 = fma_t(ekp50_002, R0_004, fma_t(ekp50_001, R0_003, ekp50_000 * R0_002));
      const T W_011 = fma_t(ekp50_002, R0_013, fma_t(ekp50_001, R0_012, ekp50_000 * R0_011));
      const T W_020 = fma_t(ekp50_002, R0_022, fma_t(ekp50_001, R0_021, ekp50_000 * R0_020));
      const T W_101 = fma_t(ekp50_002, R0_103, fma_t(ekp50_001, R0_102, ekp50_000 * R0_101));
      const T W_110 = fma_t(ekp50_002, R0_112, fma_t(ekp50_001, R0_111, ekp50_000 * R0_110));
      const T W_200 = fma_t(ekp50_002, R0_202, fma_t(ekp50_001, R0_201, ekp50_000 * R0_200));
      acc[5] += fma_t(ebx202, W_200, fma_t(ebx201, W_100, ebx200 * W_000));
      acc[11] += fma_t(ebx101 * eby101, W_110, fma_t(ebx101 * eby100, W_100, fma_t(ebx100 * eby101, W_010, ebx100 * eby100 * W_000)));
      acc[17] += fma_t(ebx101 * ebz101, W_101, fma_t(ebx101 * ebz100, W_100, fma_t(ebx100 * ebz101, W_001, ebx100 * ebz100 * W_000)));
      acc[23] += fma_t(eby202, W_020, fma_t(eby201, W_010, eby200 * W_000));
      acc[29] += fma_t(eby101 * ebz101, W_011, fma_t(eby101 * ebz100, W_010, fma_t(eby100 * ebz101, W_001, eby100 * ebz100 * W_000)));
      acc[35] += fma_t(ebz202, W_002, fma_t(ebz201, W_001, ebz200 * W_000));
    }
  }
}

// ---- class (dp|ss): 18x1 integrals, L = 3
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_dpss(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekp00_000 = ONE;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[4];
    boys_eval<T, 3>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T hp = T(0.5) * invp;
    const T ebx010 = PBx;
    const T ebx011 = hp * (ONE);
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx110 = PAx * ebx010 + ebx011;
    const T ebx111 = hp * (ebx010 + ebx100);
    const T ebx112 = (hp * T(0.5)) * (ebx011 + ebx101);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T ebx210 = PAx * ebx110 + ebx111;
    const T ebx211 = hp * (T(2) * ebx110 + ebx200);
    const T ebx212 = (hp * T(0.5)) * (T(2) * ebx111 + ebx201);
    const T ebx213 = (hp * T(0.3333333333333333)) * (T(2) * ebx112 + ebx202);
    const T eby010 = PBy;
    const T eby011 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby110 = PAy * eby010 + eby011;
    const T eby111 = hp * (eby010 + eby100);
    const T eby112 = (hp * T(0.5)) * (eby011 + eby101);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T eby210 = PAy * eby110 + eby111;
    const T eby211 = hp * (T(2) * eby110 + eby200);
    const T eby212 = (hp * T(0.5)) * (T(2) * eby111 + eby201);
    const T eby213 = (hp * T(0.3333333333333333)) * (T(2) * eby112 + eby202);
    const T ebz010 = PBz;
    const T ebz011 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz110 = PAz * ebz010 + ebz011;
    const T ebz111 = hp * (ebz010 + ebz100);
    const T ebz112 = (hp * T(0.5)) * (ebz011 + ebz101);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    const T ebz210 = PAz * ebz110 + ebz111;
    const T ebz211 = hp * (T(2) * ebz110 + ebz200);
    const T ebz212 = (hp * T(0.5)) * (T(2) * ebz111 + ebz201);
    const T ebz213 = (hp * T(0.3333333333333333)) * (T(2) * ebz112 + ebz202);
    {
      const T W_000 = ekp00_000 * R0_000;
      const T W_001 = ekp00_000 * R0_001;
      const T W_010 = ekp00_000 * R0_010;
      const T W_100 = ekp00_000 * R0_100;
      const T W_002 = ekp00_000 * R0_002;
      const T W_011 = ekp00_000 * R0_011;
      const T W_020 = ekp00_000 * R0_020;
      const T W_101 = ekp00_000 * R0_101;
      const T W_110 = ekp00_000 * R0_110;
      const T W_200 = ekp00_000 * R0_200;
      const T W_003 = ekp00_000 * R0_003;
      const T W_012 = ekp00_000 * R0_012;
      const T W_021 = ekp00_000 * R0_021;
      const T W_030 = ekp00_000 * R0_030;
      const T W_102 = ekp00_000 * R0_102;
      const T W_111 = ekp00_000 * R0_111;
      const T W_120 = ekp00_000 * R0_120;
      const T W_201 = ekp00_000 * R0_201;
      const T W_210 = ekp00_000 * R0_210;
      const T W_300 = ekp00_000 * R0_300;
      acc[0] += fma_t(ebx213, W_300, fma_t(ebx212, W_200, fma_t(ebx211, W_100, ebx210 * W_000)));
      acc[1] += fma_t(ebx202 * eby011, W_210, fma_t(ebx202 * eby010, W_200, fma_t(ebx201 * eby011, W_110, fma_t(ebx201 * eby010, W_100, fma_t(ebx200 * eby011, W_010, ebx200 * eby010 * W_000)))));
      acc[2] += fma_t(ebx202 * ebz011, W_201, fma_t(ebx202 * ebz010, W_200, fma_t(ebx201 * ebz011, W_101, fma_t(ebx201 * ebz010, W_100, fma_t(ebx200 * ebz011, W_001, ebx200 * ebz010 * W_000)))));
      acc[3] += fma_t(ebx112 * eby101, W_210, fma_t(ebx112 * eby100, W_200, fma_t(ebx111 * eby101, W_110, fma_t(ebx111 * eby100, W_100, fma_t(ebx110 * eby101, W_010, ebx110 * eby100 * W_000)))));
      acc[4] += fma_t(ebx101 * eby112, W_120, fma_t(ebx101 * eby111, W_110, fma_t(ebx101 * eby110, W_100, fma_t(ebx100 * eby112, W_020, fma_t(ebx100 * eby111, W_010, ebx100 * eby110 * W_000)))));
      acc[5] += fma_t(ebx101 * eby101 * ebz011, W_111, fma_t(ebx101 * eby101 * ebz010, W_110, fma_t(ebx101 * eby100 * ebz011, W_101, fma_t(ebx101 * eby100 * ebz010, W_100, fma_t(ebx100 * eby101 * ebz011, W_011, fma_t(ebx100 * eby101 * ebz010, W_010, fma_t(ebx100 * eby100 * ebz011, W_001, ebx100 * eby100 * ebz010 * W_000)))))));
      acc[6] += fma_t(ebx112 * ebz101, W_201, fma_t(ebx112 * ebz100, W_200, fma_t(ebx111 * ebz101, W_101, fma_t(ebx111 * ebz100, W_100, fma_t(ebx110 * ebz101, W_001, ebx110 * ebz100 * W_000)))));
      acc[7] += fma_t(ebx101 * eby011 * ebz101, W_111, fma_t(ebx101 * eby011 * ebz100, W_110, fma_t(ebx101 * eby010 * ebz101, W_101, fma_t(ebx101 * eby010 * ebz100, W_100, fma_t(ebx100 * eby011 * ebz101, W_011, fma_t(ebx100 * eby011 * ebz100, W_010, fma_t(ebx100 * eby010 * ebz101, W_001, ebx100 * eby010 * ebz100 * W_000)))))));
      acc[8] += fma_t(ebx101 * ebz112, W_102, fma_t(ebx101 * ebz111, W_101, fma_t(ebx101 * ebz110, W_100, fma_t(ebx100 * ebz112, W_002, fma_t(ebx100 * ebz111, W_001, ebx100 * ebz110 * W_000)))));
      acc[9] += fma_t(ebx011 * eby202, W_120, fma_t(ebx011 * eby201, W_110, fma_t(ebx011 * eby200, W_100, fma_t(ebx010 * eby202, W_020, fma_t(ebx010 * eby201, W_010, ebx010 * eby200 * W_000)))));
      acc[10] += fma_t(eby213, W_030, fma_t(eby212, W_020, fma_t(eby211, W_010, eby210 * W_000)));
      acc[11] += fma_t(eby202 * ebz011, W_021, fma_t(eby202 * ebz010, W_020, fma_t(eby201 * ebz011, W_011, fma_t(eby201 * ebz010, W_010, fma_t(eby200 * ebz011, W_001, eby200 * ebz010 * W_000)))));
      acc[12] += fma_t(ebx011 * eby101 * ebz101, W_111, fma_t(ebx011 * eby101 * ebz100, W_110, fma_t(ebx011 * eby100 * ebz101, W_101, fma_t(ebx011 * eby100 * ebz100, W_100, fma_t(ebx010 * eby101 * ebz101, W_011, fma_t(ebx010 * eby101 * ebz100, W_010, fma_t(ebx010 * eby100 * ebz101, W_001, ebx010 * eby100 * ebz100 * W_000)))))));
      acc[13] += fma_t(eby112 * ebz101, W_021, fma_t(eby112 * ebz100, W_020, fma_t(eby111 * ebz101, W_011, fma_t(eby111 * ebz100, W_010, fma_t(eby110 * ebz101, W_001, eby110 * ebz100 * W_000)))));
      acc[14] += fma_t(eby101 * ebz112, W_012, fma_t(eby101 * ebz111, W_011, fma_t(eby101 * ebz110, W_010, fma_t(eby100 * ebz112, W_002, fma_t(eby100 * ebz111, W_001, eby100 * ebz110 * W_000)))));
      acc[15] += fma_t(ebx011 * ebz202, W_102, fma_t(ebx011 * ebz201, W_101, fma_t(ebx011 * ebz200, W_100, fma_t(ebx010 * ebz202, W_002, fma_t(ebx010 * ebz201, W_001, ebx010 * ebz200 * W_000)))));
      acc[16] += fma_t(eby011 * ebz202, W_012, fma_t(eby011 * ebz201, W_011, fma_t(eby011 * ebz200, W_010, fma_t(eby010 * ebz202, W_002, fma_t(eby010 * ebz201, W_001, eby010 * ebz200 * W_000)))));
      acc[17] += fma_t(ebz213, W_003, fma_t(ebz212, W_002, fma_t(ebz211, W_001, ebz210 * W_000)));
    }
  }
}

// ---- class (dp|ps): 18x3 integrals, L = 4
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_dpps(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekx100 = QCx;
  const T ekx101 = hq * (ONE);
  const T eky100 = QCy;
  const T eky101 = hq * (ONE);
  const T ekz100 = QCz;
  const T ekz101 = hq * (ONE);
  const T ekp00_000 = ekx100;
  const T ekp00_100 = -(ekx101);
  const T ekp10_000 = eky100;
  const T ekp10_010 = -(eky101);
  const T ekp20_000 = ekz100;
  const T ekp20_001 = -(ekz101);
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[5];
    boys_eval<T, 4>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    scale *= m2a;
    const T R4_000 = scale * F[4];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T R3_001 = Z * R4_000;
    const T R2_002 = R3_000 + Z * R3_001;
    const T R1_003 = T(2) * R2_001 + Z * R2_002;
    const T R0_004 = T(3) * R1_002 + Z * R1_003;
    const T R0_013 = Y * R1_003;
    const T R1_012 = Y * R2_002;
    const T R0_022 = R1_002 + Y * R1_012;
    const T R2_011 = Y * R3_001;
    const T R1_021 = R2_001 + Y * R2_011;
    const T R0_031 = T(2) * R1_011 + Y * R1_021;
    const T R3_010 = Y * R4_000;
    const T R2_020 = R3_000 + Y * R3_010;
    const T R1_030 = T(2) * R2_010 + Y * R2_020;
    const T R0_040 = T(3) * R1_020 + Y * R1_030;
    const T R0_103 = X * R1_003;
    const T R0_112 = X * R1_012;
    const T R0_121 = X * R1_021;
    const T R0_130 = X * R1_030;
    const T R1_102 = X * R2_002;
    const T R0_202 = R1_002 + X * R1_102;
    const T R1_111 = X * R2_011;
    const T R0_211 = R1_011 + X * R1_111;
    const T R1_120 = X * R2_020;
    const T R0_220 = R1_020 + X * R1_120;
    const T R2_101 = X * R3_001;
    const T R1_201 = R2_001 + X * R2_101;
    const T R0_301 = T(2) * R1_101 + X * R1_201;
    const T R2_110 = X * R3_010;
    const T R1_210 = R2_010 + X * R2_110;
    const T R0_310 = T(2) * R1_110 + X * R1_210;
    const T R3_100 = X * R4_000;
    const T R2_200 = R3_000 + X * R3_100;
    const T R1_300 = T(2) * R2_100 + X * R2_200;
    const T R0_400 = T(3) * R1_200 + X * R1_300;
    const T hp = T(0.5) * invp;
    const T ebx010 = PBx;
    const T ebx011 = hp * (ONE);
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx110 = PAx * ebx010 + ebx011;
    const T ebx111 = hp * (ebx010 + ebx100);
    const T ebx112 = (hp * T(0.5)) * (ebx011 + ebx101);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T ebx210 = PAx * ebx110 + ebx111;
    const T ebx211 = hp * (T(2) * ebx110 + ebx200);
    const T ebx212 = (hp * T(0.5)) * (T(2) * ebx111 + ebx201);
    const T ebx213 = (hp * T(0.3333333333333333)) * (T(2) * ebx112 + ebx202);
    const T eby010 = PBy;
    const T eby011 = hp * (ONE);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby110 = PAy * eby010 + eby011;
    const T eby111 = hp * (eby010 + eby100);
    const T eby112 = (hp * T(0.5)) * (eby011 + eby101);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T eby210 = PAy * eby110 + eby111;
    const T eby211 = hp * (T(2) * eby110 + eby200);
    const T eby212 = (hp * T(0.5)) * (T(2) * eby111 + eby201);
    const T eby213 = (hp * T(0.3333333333333333)) * (T(2) * eby112 + eby202);
    const T ebz010 = PBz;
    const T ebz011 = hp * (ONE);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz110 = PAz * ebz010 + ebz011;
    const T ebz111 = hp * (ebz010 + ebz100);
    const T ebz112 = (hp * T(0.5)) * (ebz011 + ebz101);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    const T ebz210 = PAz * ebz110 + ebz111;
    const T ebz211 = hp * (T(2) * ebz110 + ebz200);
    const T ebz212 = (hp * T(0.5)) * (T(2) * ebz111 + ebz201);
    const T ebz213 = (hp * T(0.3333333333333333)) * (T(2) * ebz112 + ebz202);
    {
      const T W_000 = fma_t(ekp00_100, R0_100, ekp00_000 * R0_000);
      const T W_001 = fma_t(ekp00_100, R0_101, ekp00_000 * R0_001);
      const T W_010 = fma_t(ekp00_100, R0_110, ekp00_000 * R0_010);
      const T W_100 = fma_t(ekp00_100, R0_200, ekp00_000 * R0_100);
      const T W_002 = fma_t(ekp00_100, R0_102, ekp00_000 * R0_002);
      const T W_011 = fma_t(ekp00_100, R0_111, ekp00_000 * R0_011);
      const T W_020 = fma_t(ekp00_100, R0_120, ekp00_000 * R0_020);
      const T W_101 = fma_t(ekp00_100, R0_201, ekp00_000 * R0_101);
      const T W_110 = fma_t(ekp00_100, R0_210, ekp00_000 * R0_110);
      const T W_200 = fma_t(ekp00_100, R0_300, ekp00_000 * R0_200);
      const T W_003 = fma_t(ekp00_100, R0_103, ekp00_000 * R0_003);
      const T W_012 = fma_t(ekp00_100, R0_112, ekp00_000 * R0_012);
      const T W_021 = fma_t(ekp00_100, R0_121, ekp00_000 * R0_021);
      const T W_030 = fma_t(ekp00_100, R0_130, ekp00_000 * R0_030);
      const T W_102 = fma_t(ekp00_100, R0_202, ekp00_000 * R0_102);
      const T W_111 = fma_t(ekp00_100, R0_211, ekp00_000 * R0_111);
      const T W_120 = fma_t(ekp00_100, R0_220, ekp00_000 * R0_120);
      const T W_201 = fma_t(ekp00_100, R0_301, ekp00_000 * R0_201);
      const T W_210 = fma_t(ekp00_100, R0_310, ekp00_000 * R0_210);
      const T W_300 = fma_t(ekp00_100, R0_400, ekp00_000 * R0_300);
      acc[0] += fma_t(ebx213, W_300, fma_t(ebx212, W_200, fma_t(ebx211, W_100, ebx210 * W_000)));
      acc[3] += fma_t(ebx202 * eby011, W_210, fma_t(ebx202 * eby010, W_200, fma_t(ebx201 * eby011, W_110, fma_t(ebx201 * eby010, W_100, fma_t(ebx200 * eby011, W_010, ebx200 * eby010 * W_000)))));
      acc[6] += fma_t(ebx202 * ebz011, W_201, fma_t(ebx202 * ebz010, W_200, fma_t(ebx201 * ebz011, W_101, fma_t(ebx201 * ebz010, W_100, fma_t(ebx200 * ebz011, W_001, ebx200 * ebz010 * W_000)))));
      acc[9] += fma_t(ebx112 * eby101, W_210, fma_t(ebx112 * eby100, W_200, fma_t(ebx111 * eby101, W_110, fma_t(ebx111 * eby100, W_100, fma_t(ebx110 * eby101, W_010, ebx110 * eby100 * W_000)))));
      acc[12] += fma_t(ebx101 * eby112, W_120, fma_t(ebx101 * eby111, W_110, fma_t(ebx101 * eby110, W_100, fma_t(ebx100 * eby112, W_020, fma_t(ebx100 * eby111, W_010, ebx100 * eby110 * W_000)))));
      acc[15] += fma_t(ebx101 * eby101 * ebz011, W_111, fma_t(ebx101 * eby101 * ebz010, W_110, fma_t(ebx101 * eby100 * ebz011, W_101, fma_t(ebx101 * eby100 * ebz010, W_100, fma_t(ebx100 * eby101 * ebz011, W_011, fma_t(ebx100 * eby101 * ebz010, W_010, fma_t(ebx100 * eby100 * ebz011, W_001, ebx100 * eby100 * ebz010 * W_000)))))));
      acc[18] += fma_t(ebx112 * ebz101, W_201, fma_t(ebx112 * ebz100, W_200, fma_t(ebx111 * ebz101, W_101, fma_t(ebx111 * ebz100, W_100, fma_t(ebx110 * ebz101, W_001, ebx110 * ebz100 * W_000)))));
      acc[21] += fma_t(ebx101 * eby011 * ebz101, W_111, fma_t(ebx101 * eby011 * ebz100, W_110, fma_t(ebx101 * eby010 * ebz101, W_101, fma_t(ebx101 * eby010 * ebz100, W_100, fma_t(ebx100 * eby011 * ebz101, W_011, fma_t(ebx100 * eby011 * ebz100, W_010, fma_t(ebx100 * eby010 * ebz101, W_001, ebx100 * eby010 * ebz100 * W_000)))))));
      acc[24] += fma_t(ebx101 * ebz112, W_102, fma_t(ebx101 * ebz111, W_101, fma_t(ebx101 * ebz110, W_100, fma_t(ebx100 * ebz112, W_002, fma_t(ebx100 * ebz111, W_001, ebx100 * ebz110 * W_000)))));
      acc[27] += fma_t(ebx011 * eby202, W_120, fma_t(ebx011 * eby201, W_110, fma_t(ebx011 * eby200, W_100, fma_t(ebx010 * eby202, W_020, fma_t(ebx010 * eby201, W_010, ebx010 * eby200 * W_000)))));
      acc[30] += fma_t(eby213, W_030, fma_t(eby212, W_020, fma_t(eby211, W_010, eby210 * W_000)));
      acc[33] += fma_t(eby202 * ebz011, W_021, fma_t(eby202 * ebz010, W_020, fma_t(eby201 * ebz011, W_011, fma_t(eby201 * ebz010, W_010, fma_t(eby200 * ebz011, W_001, eby200 * ebz010 * W_000)))));
      acc[36] += fma_t(ebx011 * eby101 * ebz101, W_111, fma_t(ebx011 * eby101 * ebz100, W_110, fma_t(ebx011 * eby100 * ebz101, W_101, fma_t(ebx011 * eby100 * ebz100, W_100, fma_t(ebx010 * eby101 * ebz101, W_011, fma_t(ebx010 * eby101 * ebz100, W_010, fma_t(ebx010 * eby100 * ebz101, W_001, ebx010 * eby100 * ebz100 * W_000)))))));
      acc[39] += fma_t(eby112 * ebz101, W_021, fma_t(eby112 * ebz100, W_020, fma_t(eby111 * ebz101, W_011, fma_t(eby111 * ebz100, W_010, fma_t(eby110 * ebz101, W_001, eby110 * ebz100 * W_000)))));
      acc[42] += fma_t(eby101 * ebz112, W_012, fma_t(eby101 * ebz111, W_011, fma_t(eby101 * ebz110, W_010, fma_t(eby100 * ebz112, W_002, fma_t(eby100 * ebz111, W_001, eby100 * ebz110 * W_000)))));
      acc[45] += fma_t(ebx011 * ebz202, W_102, fma_t(ebx011 * ebz201, W_101, fma_t(ebx011 * ebz200, W_100, fma_t(ebx010 * ebz202, W_002, fma_t(ebx010 * ebz201, W_001, ebx010 * ebz200 * W_000)))));
      acc[48] += fma_t(eby011 * ebz202, W_012, fma_t(eby011 * ebz201, W_011, fma_t(eby011 * ebz200, W_010, fma_t(eby010 * ebz202, W_002, fma_t(eby010 * ebz201, W_001, eby010 * ebz200 * W_000)))));
      acc[51] += fma_t(ebz213, W_003, fma_t(ebz212, W_002, fma_t(ebz211, W_001, ebz210 * W_000)));
    }
    {
      const T W_000 = fma_t(ekp10_010, R0_010, ekp10_000 * R0_000);
      const T W_001 = fma_t(ekp10_010, R0_011, ekp10_000 * R0_001);
      const T W_010 = fma_t(ekp10_010, R0_020, ekp10_000 * R0_010);
      const T W_100 = fma_t(ekp10_010, R0_110, ekp10_000 * R0_100);
      const T W_002 = fma_t(ekp10_010, R0_012, ekp10_000 * R0_002);
      const T W_011 = fma_t(ekp10_010, R0_021, ekp10_000 * R0_011);
      const T W_020 = fma_t(ekp10_010, R0_030, ekp10_000 * R0_020);
      const T W_101 = fma_t(ekp10_010, R0_111, ekp10_000 * R0_101);
      const T W_110 = fma_t(ekp10_010, R0_120, ekp10_000 * R0_110);
      const T W_200 = fma_t(ekp10_010, R0_210, ekp10_000 * R0_200);
      const T W_003 = fma_t(ekp10_010, R0_013, ekp10_000 * R0_003);
      const T W_012 = fma_t(ekp10_010, R0_022, ekp10_000 * R0_012);
      const T W_021 = fma_t(ekp10_010, R0_031, ekp10_000 * R0_021);
      const T W_030 = fma_t(ekp10_010, R0_040, ekp10_000 * R0_030);
      const T W_102 = fma_t(ekp10_010, R0_112, ekp10_000 * R0_102);
      const T W_111 = fma_t(ekp10_010, R0_121, ekp10_000 * R0_111);
      const T W_120 = fma_t(ekp10_010, R0_130, ekp10_000 * R0_120);
      const T W_201 = fma_t(ekp10_010, R0_211, ekp10_000 * R0_201);
      const T W_210 = fma_t(ekp10_010, R0_220, ekp10_000 * R0_210);
      const T W_300 = fma_t(ekp10_010, R0_310, ekp10_000 * R0_300);
      acc[1] += fma_t(ebx213, W_300, fma_t(ebx212, W_200, fma_t(ebx211, W_100, ebx210 * W_000)));
      acc[4] += fma_t(ebx202 * eby011, W_210, fma_t(ebx202 * eby010, W_200, fma_t(ebx201 * eby011, W_110, fma_t(ebx201 * eby010, W_100, fma_t(ebx200 * eby011, W_010, ebx200 * eby010 * W_000)))));
      acc[7] += fma_t(ebx202 * ebz011, W_201, fma_t(ebx202 * ebz010, W_200, fma_t(ebx201 * ebz011, W_101, fma_t(ebx201 * ebz010, W_100, fma_t(ebx200 * ebz011, W_001, ebx200 * ebz010 * W_000)))));
      acc[10] += fma_t(ebx112 * eby101, W_210, fma_t(ebx112 * eby100, W_200, fma_t(ebx111 * eby101, W_110, fma_t(ebx111 * eby100, W_100, fma_t(ebx110 * eby101, W_010, ebx110 * eby100 * W_000)))));
      acc[13] += fma_t(ebx101 * eby112, W_120, fma_t(ebx101 * eby111, W_110, fma_t(ebx101 * eby110, W_100, fma_t(ebx100 * eby112, W_020, fma_t(ebx100 * eby111, W_010, ebx100 * eby110 * W_000)))));
      acc[16] += fma_t(ebx101 * eby101 * ebz011, W_111, fma_t(ebx101 * eby101 * ebz010, W_110, fma_t(ebx101 * eby100 * ebz011, W_101, fma_t(ebx101 * eby100 * ebz010, W_100, fma_t(ebx100 * eby101 * ebz011, W_011, fma_t(ebx100 * eby101 * ebz010, W_010, fma_t(ebx100 * eby100 * ebz011, W_001, ebx100 * eby100 * ebz010 * W_000)))))));
      acc[19] += fma_t(ebx112 * ebz101, W_201, fma_t(ebx112 * ebz100, W_200, fma_t(ebx111 * ebz101, W_101, fma_t(ebx111 * ebz100, W_100, fma_t(ebx110 * ebz101, W_001, ebx110 * ebz100 * W_000)))));
      acc[22] += fma_t(ebx101 * eby011 * ebz101, W_111, fma_t(ebx101 * eby011 * ebz100, W_110, fma_t(ebx101 * eby010 * ebz101, W_101, fma_t(ebx101 * eby010 * ebz100, W_100, fma_t(ebx100 * eby011 * ebz101, W_011, fma_t(ebx100 * eby011 * ebz100, W_010, fma_t(ebx100 * eby010 * ebz101, W_001, ebx100 * eby010 * ebz100 * W_000)))))));
      acc[25] += fma_t(ebx101 * ebz112, W_102, fma_t(ebx101 * ebz111, W_101, fma_t(ebx101 * ebz110, W_100, fma_t(ebx100 * ebz112, W_002, fma_t(ebx100 * ebz111, W_001, ebx100 * ebz110 * W_000)))));
      acc[28] += fma_t(ebx011 * eby202, W_120, fma_t(ebx011 * eby201, W_110, fma_t(ebx011 * eby200, W_100, fma_t(ebx010 * eby202, W_020, fma_t(ebx010 * eby201, W_010, ebx010 * eby200 * W_000)))));
      acc[31] += fma_t(eby213, W_030, fma_t(eby212, W_020, fma_t(eby211, W_010, eby210 * W_000)));
      acc[34] += fma_t(eby202 * ebz011, W_021, fma_t(eby202 * ebz010, W_020, fma_t(eby201 * ebz011, W_011, fma_t(eby201 * ebz010, W_010, fma_t(eby200 * ebz011, W_001, eby200 * ebz010 * W_000)))));
      acc[37] += fma_t(ebx011 * eby101 * ebz101, W_111, fma_t(ebx011 * eby101 * ebz100, W_110, fma_t(ebx011 * eby100 * ebz101, W_101, fma_t(ebx011 * eby100 * ebz100, W_100, fma_t(ebx010 * eby101 * ebz101, W_011, fma_t(ebx010 * eby101 * ebz100, W_010, fma_t(ebx010 * eby100 * ebz101, W_001, ebx010 * eby100 * ebz100 * W_000)))))));
      acc[40] += fma_t(eby112 * ebz101, W_021, fma_t(eby112 * ebz100, W_020, fma_t(eby111 * ebz101, W_011, fma_t(eby111 * ebz100, W_010, fma_t(eby110 * ebz101, W_001, eby110 * ebz100 * W_000)))));
      acc[43] += fma_t(eby101 * ebz112, W_012, fma_t(eby101 * ebz111, W_011, fma_t(eby101 * ebz110, W_010, fma_t(eby100 * ebz112, W_002, fma_t(eby100 * ebz111, W_001, eby100 * ebz110 * W_000)))));
      acc[46] += fma_t(ebx011 * ebz202, W_102, fma_t(ebx011 * ebz201, W_101, fma_t(ebx011 * ebz200, W_100, fma_t(ebx010 * ebz202, W_002, fma_t(ebx010 * ebz201, W_001, ebx010 * ebz200 * W_000)))));
      acc[49] += fma_t(eby011 * ebz202, W_012, fma_t(eby011 * ebz201, W_011, fma_t(eby011 * ebz200, W_010, fma_t(eby010 * ebz202, W_002, fma_t(eby010 * ebz201, W_001, eby010 * ebz200 * W_000)))));
      acc[52] += fma_t(ebz213, W_003, fma_t(ebz212, W_002, fma_t(ebz211, W_001, ebz210 * W_000)));
    }
    {
      const T W_000 = fma_t(ekp20_001, R0_001, ekp20_000 * R0_000);
      const T W_001 = fma_t(ekp20_001, R0_002, ekp20_000 * R0_001);
      const T W_010 = fma_t(ekp20_001, R0_011, ekp20_000 * R0_010);
      const T W_100 = fma_t(ekp20_001, R0_101, ekp20_000 * R0_100);
      const T W_002 = fma_t(ekp20_001, R0_003, ekp20_000 * R0_002);
      const T W_011 = fma_t(ekp20_001, R0_012, ekp20_000 * R0_011);
      const T W_020 = fma_t(ekp20_001, R0_021, ekp20_000 * R0_020);
      const T W_101 = fma_t(ekp20_001, R0_102, ekp20_000 * R0_101);
      const T W_110 = fma_t(ekp20_001, R0_111, ekp20_000 * R0_110);
      const T W_200 = fma_t(ekp20_001, R0_201, ekp20_000 * R0_200);
      const T W_003 = fma_t(ekp20_001, R0_004, ekp20_000 * R0_003);
      const T W_012 = fma_t(ekp20_001, R0_013, ekp20_000 * R0_012);
      const T W_021 = fma_t(ekp20_001, R0_022, ekp20_000 * R0_021);
      const T W_030 = fma_t(ekp20_001, R0_031, ekp20_000 * R0_030);
      const T W_102 = fma_t(ekp20_001, R0_103, ekp20_000 * R0_102);
      const T W_111 = fma_t(ekp20_001, R0_112, ekp20_000 * R0_111);
      const T W_120 = fma_t(ekp20_001, R0_121, ekp20_000 * R0_120);
      const T W_201 = fma_t(ekp20_001, R0_202, ekp20_000 * R0_201);
      const T W_210 = fma_t(ekp20_001, R0_211, ekp20_000 * R0_210);
      const T W_300 = fma_t(ekp20_001, R0_301, ekp20_000 * R0_300);
      acc[2] += fma_t(ebx213, W_300, fma_t(ebx212, W_200, fma_t(ebx211, W_100, ebx210 * W_000)));
      acc[5] += fma_t(ebx202 * eby011, W_210, fma_t(ebx202 * eby010, W_200, fma_t(ebx201 * eby011, W_110, fma_t(ebx201 * eby010, W_100, fma_t(ebx200 * eby011, W_010, ebx200 * eby010 * W_000)))));
      acc[8] += fma_t(ebx202 * ebz011, W_201, fma_t(ebx202 * ebz010, W_200, fma_t(ebx201 * ebz011, W_101, fma_t(ebx201 * ebz010, W_100, fma_t(ebx200 * ebz011, W_001, ebx200 * ebz010 * W_000)))));
      acc[11] += fma_t(ebx112 * eby101, W_210, fma_t(ebx112 * eby100, W_200, fma_t(ebx111 * eby101, W_110, fma_t(ebx111 * eby100, W_100, fma_t(ebx110 * eby101, W_010, ebx110 * eby100 * W_000)))));
      acc[14] += fma_t(ebx101 * eby112, W_120, fma_t(ebx101 * eby111, W_110, fma_t(ebx101 * eby110, W_100, fma_t(ebx100 * eby112, W_020, fma_t(ebx100 * eby111, W_010, ebx100 * eby110 * W_000)))));
      acc[17] += fma_t(ebx101 * eby101 * ebz011, W_111, fma_t(ebx101 * eby101 * ebz010, W_110, fma_t(ebx101 * eby100 * ebz011, W_101, fma_t(ebx101 * eby100 * ebz010, W_100, fma_t(ebx100 * eby101 * ebz011, W_011, fma_t(ebx100 * eby101 * ebz010, W_010, fma_t(ebx100 * eby100 * ebz011, W_001, ebx100 * eby100 * ebz010 * W_000)))))));
      acc[20] += fma_t(ebx112 * ebz101, W_201, fma_t(ebx112 * ebz100, W_200, fma_t(ebx111 * ebz101, W_101, fma_t(ebx111 * ebz100, W_100, fma_t(ebx110 * ebz101, W_001, ebx110 * ebz100 * W_000)))));
      acc[23] += fma_t(ebx101 * eby011 * ebz101, W_111, fma_t(ebx101 * eby011 * ebz100, W_110, fma_t(ebx101 * eby010 * ebz101, W_101, fma_t(ebx101 * eby010 * ebz100, W_100, fma_t(ebx100 * eby011 * ebz101, W_011, fma_t(ebx100 * eby011 * ebz100, W_010, fma_t(ebx100 * eby010 * ebz101, W_001, ebx100 * eby010 * ebz100 * W_000)))))));
      acc[26] += fma_t(ebx101 * ebz112, W_102, fma_t(ebx101 * ebz111, W_101, fma_t(ebx101 * ebz110, W_100, fma_t(ebx100 * ebz112, W_002, fma_t(ebx100 * ebz111, W_001, ebx100 * ebz110 * W_000)))));
      acc[29] += fma_t(ebx011 * eby202, W_120, fma_t(ebx011 * eby201, W_110, fma_t(ebx011 * eby200, W_100, fma_t(ebx010 * eby202, W_020, fma_t(ebx010 * eby201, W_010, ebx010 * eby200 * W_000)))));
      acc[32] += fma_t(eby213, W_030, fma_t(eby212, W_020, fma_t(eby211, W_010, eby210 * W_000)));
      acc[35] += fma_t(eby202 * ebz011, W_021, fma_t(eby202 * ebz010, W_020, fma_t(eby201 * ebz011, W_011, fma_t(eby201 * ebz010, W_010, fma_t(eby200 * ebz011, W_001, eby200 * ebz010 * W_000)))));
      acc[38] += fma_t(ebx011 * eby101 * ebz101, W_111, fma_t(ebx011 * eby101 * ebz100, W_110, fma_t(ebx011 * eby100 * ebz101, W_101, fma_t(ebx011 * eby100 * ebz100, W_100, fma_t(ebx010 * eby101 * ebz101, W_011, fma_t(ebx010 * eby101 * ebz100, W_010, fma_t(ebx010 * eby100 * ebz101, W_001, ebx010 * eby100 * ebz100 * W_000)))))));
      acc[41] += fma_t(eby112 * ebz101, W_021, fma_t(eby112 * ebz100, W_020, fma_t(eby111 * ebz101, W_011, fma_t(eby111 * ebz100, W_010, fma_t(eby110 * ebz101, W_001, eby110 * ebz100 * W_000)))));
      acc[44] += fma_t(eby101 * ebz112, W_012, fma_t(eby101 * ebz111, W_011, fma_t(eby101 * ebz110, W_010, fma_t(eby100 * ebz112, W_002, fma_t(eby100 * ebz111, W_001, eby100 * ebz110 * W_000)))));
      acc[47] += fma_t(ebx011 * ebz202, W_102, fma_t(ebx011 * ebz201, W_101, fma_t(ebx011 * ebz200, W_100, fma_t(ebx010 * ebz202, W_002, fma_t(ebx010 * ebz201, W_001, ebx010 * ebz200 * W_000)))));
      acc[50] += fma_t(eby011 * ebz202, W_012, fma_t(eby011 * ebz201, W_011, fma_t(eby011 * ebz200, W_010, fma_t(eby010 * ebz202, W_002, fma_t(eby010 * ebz201, W_001, eby010 * ebz200 * W_000)))));
      acc[53] += fma_t(ebz213, W_003, fma_t(ebz212, W_002, fma_t(ebz211, W_001, ebz210 * W_000)));
    }
  }
}

// ---- class (dd|ss): 36x1 integrals, L = 4
template <typename T, typename Acc>
__device__ __forceinline__ void eri_ketprim_ddss(const T* __restrict__ sb, int nbra, int bstep,
    const T q, const T invq, const T Qx, const T Qy, const T Qz,
    const T QCx, const T QCy, const T QCz, const T QDx, const T QDy, const T QDz,
    const T Kcd, const T* __restrict__ boys, Acc& acc) {
  const T ONE = T(1);
  (void)QCx; (void)QCy; (void)QCz; (void)QDx; (void)QDy; (void)QDz;
  const T hq = T(0.5) * invq;
  const T ekp00_000 = ONE;
  #pragma unroll 1
  for (int kb = 0; kb < nbra; ++kb) {
    BraPrim<T> bp;
    load_bra_prim(sb + kb * bstep, bp);
    const T p = bp.p, invp = bp.invp, Px = bp.Px, Py = bp.Py, Pz = bp.Pz;
    const T PAx = bp.PAx, PAy = bp.PAy, PAz = bp.PAz;
    const T PBx = bp.PBx, PBy = bp.PBy, PBz = bp.PBz;
    const T Kab = bp.K;
    const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    const T ppq = p + q;
    const T rs = rsqrt_t(ppq);
    const T alpha = p * q * (rs * rs);
    const T Tb = alpha * (X * X + Y * Y + Z * Z);
    const T pref = Kab * Kcd * rs;   // K holds sqrt(2 pi^2.5) c c exp(-mu R^2) / p
    T F[5];
    boys_eval<T, 4>(Tb, boys, F);
    const T m2a = T(-2) * alpha;
    T scale = pref;
    const T R0_000 = scale * F[0];
    scale *= m2a;
    const T R1_000 = scale * F[1];
    scale *= m2a;
    const T R2_000 = scale * F[2];
    scale *= m2a;
    const T R3_000 = scale * F[3];
    scale *= m2a;
    const T R4_000 = scale * F[4];
    const T R0_001 = Z * R1_000;
    const T R0_010 = Y * R1_000;
    const T R0_100 = X * R1_000;
    const T R1_001 = Z * R2_000;
    const T R0_002 = R1_000 + Z * R1_001;
    const T R0_011 = Y * R1_001;
    const T R1_010 = Y * R2_000;
    const T R0_020 = R1_000 + Y * R1_010;
    const T R0_101 = X * R1_001;
    const T R0_110 = X * R1_010;
    const T R1_100 = X * R2_000;
    const T R0_200 = R1_000 + X * R1_100;
    const T R2_001 = Z * R3_000;
    const T R1_002 = R2_000 + Z * R2_001;
    const T R0_003 = T(2) * R1_001 + Z * R1_002;
    const T R0_012 = Y * R1_002;
    const T R1_011 = Y * R2_001;
    const T R0_021 = R1_001 + Y * R1_011;
    const T R2_010 = Y * R3_000;
    const T R1_020 = R2_000 + Y * R2_010;
    const T R0_030 = T(2) * R1_010 + Y * R1_020;
    const T R0_102 = X * R1_002;
    const T R0_111 = X * R1_011;
    const T R0_120 = X * R1_020;
    const T R1_101 = X * R2_001;
    const T R0_201 = R1_001 + X * R1_101;
    const T R1_110 = X * R2_010;
    const T R0_210 = R1_010 + X * R1_110;
    const T R2_100 = X * R3_000;
    const T R1_200 = R2_000 + X * R2_100;
    const T R0_300 = T(2) * R1_100 + X * R1_200;
    const T R3_001 = Z * R4_000;
    const T R2_002 = R3_000 + Z * R3_001;
    const T R1_003 = T(2) * R2_001 + Z * R2_002;
    const T R0_004 = T(3) * R1_002 + Z * R1_003;
    const T R0_013 = Y * R1_003;
    const T R1_012 = Y * R2_002;
    const T R0_022 = R1_002 + Y * R1_012;
    const T R2_011 = Y * R3_001;
    const T R1_021 = R2_001 + Y * R2_011;
    const T R0_031 = T(2) * R1_011 + Y * R1_021;
    const T R3_010 = Y * R4_000;
    const T R2_020 = R3_000 + Y * R3_010;
    const T R1_030 = T(2) * R2_010 + Y * R2_020;
    const T R0_040 = T(3) * R1_020 + Y * R1_030;
    const T R0_103 = X * R1_003;
    const T R0_112 = X * R1_012;
    const T R0_121 = X * R1_021;
    const T R0_130 = X * R1_030;
    const T R1_102 = X * R2_002;
    const T R0_202 = R1_002 + X * R1_102;
    const T R1_111 = X * R2_011;
    const T R0_211 = R1_011 + X * R1_111;
    const T R1_120 = X * R2_020;
    const T R0_220 = R1_020 + X * R1_120;
    const T R2_101 = X * R3_001;
    const T R1_201 = R2_001 + X * R2_101;
    const T R0_301 = T(2) * R1_101 + X * R1_201;
    const T R2_110 = X * R3_010;
    const T R1_210 = R2_010 + X * R2_110;
    const T R0_310 = T(2) * R1_110 + X * R1_210;
    const T R3_100 = X * R4_000;
    const T R2_200 = R3_000 + X * R3_100;
    const T R1_300 = T(2) * R2_100 + X * R2_200;
    const T R0_400 = T(3) * R1_200 + X * R1_300;
    const T hp = T(0.5) * invp;
    const T ebx010 = PBx;
    const T ebx011 = hp * (ONE);
    const T ebx020 = PBx * ebx010 + ebx011;
    const T ebx021 = hp * (T(2) * ebx010);
    const T ebx022 = (hp * T(0.5)) * (T(2) * ebx011);
    const T ebx100 = PAx;
    const T ebx101 = hp * (ONE);
    const T ebx110 = PAx * ebx010 + ebx011;
    const T ebx111 = hp * (ebx010 + ebx100);
    const T ebx112 = (hp * T(0.5)) * (ebx011 + ebx101);
    const T ebx120 = PAx * ebx020 + ebx021;
    const T ebx121 = hp * (ebx020 + T(2) * ebx110);
    const T ebx122 = (hp * T(0.5)) * (ebx021 + T(2) * ebx111);
    const T ebx123 = (hp * T(0.3333333333333333)) * (ebx022 + T(2) * ebx112);
    const T ebx200 = PAx * ebx100 + ebx101;
    const T ebx201 = hp * (T(2) * ebx100);
    const T ebx202 = (hp * T(0.5)) * (T(2) * ebx101);
    const T ebx210 = PAx * ebx110 + ebx111;
    const T ebx211 = hp * (T(2) * ebx110 + ebx200);
    const T ebx212 = (hp * T(0.5)) * (T(2) * ebx111 + ebx201);
    const T ebx213 = (hp * T(0.3333333333333333)) * (T(2) * ebx112 + ebx202);
    const T ebx220 = PAx * ebx120 + ebx121;
    const T ebx221 = hp * (T(2) * ebx120 + T(2) * ebx210);
    const T ebx222 = (hp * T(0.5)) * (T(2) * ebx121 + T(2) * ebx211);
    const T ebx223 = (hp * T(0.3333333333333333)) * (T(2) * ebx122 + T(2) * ebx212);
    const T ebx224 = (hp * T(0.25)) * (T(2) * ebx123 + T(2) * ebx213);
    const T eby010 = PBy;
    const T eby011 = hp * (ONE);
    const T eby020 = PBy * eby010 + eby011;
    const T eby021 = hp * (T(2) * eby010);
    const T eby022 = (hp * T(0.5)) * (T(2) * eby011);
    const T eby100 = PAy;
    const T eby101 = hp * (ONE);
    const T eby110 = PAy * eby010 + eby011;
    const T eby111 = hp * (eby010 + eby100);
    const T eby112 = (hp * T(0.5)) * (eby011 + eby101);
    const T eby120 = PAy * eby020 + eby021;
    const T eby121 = hp * (eby020 + T(2) * eby110);
    const T eby122 = (hp * T(0.5)) * (eby021 + T(2) * eby111);
    const T eby123 = (hp * T(0.3333333333333333)) * (eby022 + T(2) * eby112);
    const T eby200 = PAy * eby100 + eby101;
    const T eby201 = hp * (T(2) * eby100);
    const T eby202 = (hp * T(0.5)) * (T(2) * eby101);
    const T eby210 = PAy * eby110 + eby111;
    const T eby211 = hp * (T(2) * eby110 + eby200);
    const T eby212 = (hp * T(0.5)) * (T(2) * eby111 + eby201);
    const T eby213 = (hp * T(0.3333333333333333)) * (T(2) * eby112 + eby202);
    const T eby220 = PAy * eby120 + eby121;
    const T eby221 = hp * (T(2) * eby120 + T(2) * eby210);
    const T eby222 = (hp * T(0.5)) * (T(2) * eby121 + T(2) * eby211);
    const T eby223 = (hp * T(0.3333333333333333)) * (T(2) * eby122 + T(2) * eby212);
    const T eby224 = (hp * T(0.25)) * (T(2) * eby123 + T(2) * eby213);
    const T ebz010 = PBz;
    const T ebz011 = hp * (ONE);
    const T ebz020 = PBz * ebz010 + ebz011;
    const T ebz021 = hp * (T(2) * ebz010);
    const T ebz022 = (hp * T(0.5)) * (T(2) * ebz011);
    const T ebz100 = PAz;
    const T ebz101 = hp * (ONE);
    const T ebz110 = PAz * ebz010 + ebz011;
    const T ebz111 = hp * (ebz010 + ebz100);
    const T ebz112 = (hp * T(0.5)) * (ebz011 + ebz101);
    const T ebz120 = PAz * ebz020 + ebz021;
    const T ebz121 = hp * (ebz020 + T(2) * ebz110);
    const T ebz122 = (hp * T(0.5)) * (ebz021 + T(2) * ebz111);
    const T ebz123 = (hp * T(0.3333333333333333)) * (ebz022 + T(2) * ebz112);
    const T ebz200 = PAz * ebz100 + ebz101;
    const T ebz201 = hp * (T(2) * ebz100);
    const T ebz202 = (hp * T(0.5)) * (T(2) * ebz101);
    const T ebz210 = PAz * ebz110 + ebz111;
    const T ebz211 = hp * (T(2) * ebz110 + ebz200);
    const T ebz212 = (hp * T(0.5)) * (T(2) * ebz111 + ebz201);
    const T ebz213 = (hp * T(0.3333333333333333)) * (T(2) * ebz112 + ebz202);
    const T ebz220 = PAz * ebz120 + ebz121;
    const T ebz221 = hp * (T(2) * ebz120 + T(2) * ebz210);
    const T ebz222 = (hp * T(0.5)) * (T(2) * ebz121 + T(2) * ebz211);
    const T ebz223 = (hp * T(0.3333333333333333)) * (T(2) * ebz122 + T(2) * ebz212);
    const T ebz224 = (hp * T(0.25)) * (T(2) * ebz123 + T(2) * ebz213);
    {
      const T W_000 = ekp00_000 * R0_000;
      const T W_001 = ekp00_000 * R0_001;
      const T W_010 = ekp00_000 * R0_010;
      const T W_100 = ekp00_000 * R0_100;
      const T W_002 = ekp00_000 * R0_002;
      const T W_011 = ekp00_000 * R0_011;
      const T W_020 = ekp00_000 * R0_020;
      const T W_101 = ekp00_000 * R0_101;
      const T W_110 = ekp00_000 * R0_110;
      const T W_200 = ekp00_000 * R0_200;
      const T W_003 = ekp00_000 * R0_003;
      const T W_012 = ekp00_000 * R0_012;
      const T W_021 = ekp00_000 * R0_021;
      const T W_030 = ekp00_000 * R0_030;
      const T W_102 = ekp00_000 * R0_102;
      const T W_111 = ekp00_000 * R0_111;
      const T W_120 = ekp00_000 * R0_120;
      const T W_201 = ekp00_000 * R0_201;
      const T W_210 = ekp00_000 * R0_210;
      const T W_300 = ekp00_000 * R0_300;
      const T W_004 = ekp00_000 * R0_004;
      const T W_013 = ekp00_000 * R0_013;
      const T W_022 = ekp00_000 * R0_022;
      const T W_031 = ekp00_000 * R0_031;
      const T W_040 = ekp00_000 * R0_040;
      const T W_103 = ekp00_000 * R0_103;
      const T W_112 = ekp00_000 * R0_112;
      const T W_121 = ekp00_000 * R0_121;
      const T W_130 = ekp00_000 * R0_130;
      const T W_202 = ekp00_000 * R0_202;
      const T W_211 = ekp00_000 * R0_211;
      const T W_220 = ekp00_000 * R0_220;
      const T W_301 = ekp00_000 * R0_301;
      const T W_310 = ekp00_000 * R0_310;
      const T W_400 = ekp00_000 * R0_400;
      acc[0] += fma_t(ebx224, W_400, fma_t(ebx223, W_300, fma_t(ebx222, W_200, fma_t(ebx221, W_100, ebx220 * W_000))));
      acc[1] += fma_t(ebx213 * eby011, W_310, fma_t(ebx213 * eby010, W_300, fma_t(ebx212 * eby011, W_210, fma_t(ebx212 * eby010, W_200, fma_t(ebx211 * eby011, W_110, fma_t(ebx211 * eby010, W_100, fma_t(ebx210 * eby011, W_010, ebx210 * eby010 * W_000)))))));
      acc[2] += fma_t(ebx213 * ebz011, W_301, fma_t(ebx213 * ebz010, W_300, fma_t(ebx212 * ebz011, W_201, fma_t(ebx212 * ebz010, W_200, fma_t(ebx211 * ebz011, W_101, fma_t(ebx211 * ebz010, W_100, fma_t(ebx210 * ebz011, W_001, ebx210 * ebz010 * W_000)))))));
      acc[3] += fma_t(ebx202 * eby022, W_220, fma_t(ebx202 * eby021, W_210, fma_t(ebx202 * eby020, W_200, fma_t(ebx201 * eby022, W_120, fma_t(ebx201 * eby021, W_110, fma_t(ebx201 * eby020, W_100, fma_t(ebx200 * eby022, W_020, fma_t(ebx200 * eby021, W_010, ebx200 * eby020 * W_000))))))));
      acc[4] += fma_t(ebx202 * eby011 * ebz011, W_211, fma_t(ebx202 * eby011 * ebz010, W_210, fma_t(ebx202 * eby010 * ebz011, W_201, fma_t(ebx202 * eby010 * ebz010, W_200, fma_t(ebx201 * eby011 * ebz011, W_111, fma_t(ebx201 * eby011 * ebz010, W_110, fma_t(ebx201 * eby010 * ebz011, W_101, fma_t(ebx201 * eby010 * ebz010, W_100, fma_t(ebx200 * eby011 * ebz011, W_011, fma_t(ebx200 * eby011 * ebz010, W_010, fma_t(ebx200 * eby010 * ebz011, W_001, ebx200 * eby010 * ebz010 * W_000)))))))))));
      acc[5] += fma_t(ebx202 * ebz022, W_202, fma_t(ebx202 * ebz021, W_201, fma_t(ebx202 * ebz020, W_200, fma_t(ebx201 * ebz022, W_102, fma_t(ebx201 * ebz021, W_101, fma_t(ebx201 * ebz020, W_100, fma_t(ebx200 * ebz022, W_002, fma_t(ebx200 * ebz021, W_001, ebx200 * ebz020 * W_000))))))));
      acc[6] += fma_t(ebx123 * eby101, W_310, fma_t(ebx123 * eby100, W_300, fma_t(ebx122 * eby101, W_210, fma_t(ebx122 * eby100, W_200, fma_t(ebx121 * eby101, W_110, fma_t(ebx121 * eby100, W_100, fma_t(ebx120 * eby101, W_010, ebx120 * eby100 * W_000)))))));
      acc[7] += fma_t(ebx112 * eby112, W_220, fma_t(ebx112 * eby111, W_210, fma_t(ebx112 * eby110, W_200, fma_t(ebx111 * eby112, W_120, fma_t(ebx111 * eby111, W_110, fma_t(ebx111 * eby110, W_100, fma_t(ebx110 * eby112, W_020, fma_t(ebx110 * eby111, W_010, ebx110 * eby110 * W_000))))))));
      acc[8] += fma_t(ebx112 * eby101 * ebz011, W_211, fma_t(ebx112 * eby101 * ebz010, W_210, fma_t(ebx112 * eby100 * ebz011, W_201, fma_t(ebx112 * eby100 * ebz010, W_200, fma_t(ebx111 * eby101 * ebz011, W_111, fma_t(ebx111 * eby101 * ebz010, W_110, fma_t(ebx111 * eby100 * ebz011, W_101, fma_t(ebx111 * eby100 * ebz010, W_100, fma_t(ebx110 * eby101 * ebz011, W_011, fma_t(ebx110 * eby101 * ebz010, W_010, fma_t(ebx110 * eby100 * ebz011, W_001, ebx110 * eby100 * ebz010 * W_000)))))))))));
      acc[9] += fma_t(ebx101 * eby123, W_130, fma_t(ebx101 * eby122, W_120, fma_t(ebx101 * eby121, W_110, fma_t(ebx101 * eby120, W_100, fma_t(ebx100 * eby123, W_030, fma_t(ebx100 * eby122, W_020, fma_t(ebx100 * eby121, W_010, ebx100 * eby120 * W_000)))))));
      acc[10] += fma_t(ebx101 * eby112 * ebz011, W_121, fma_t(ebx101 * eby112 * ebz010, W_120, fma_t(ebx101 * eby111 * ebz011, W_111, fma_t(ebx101 * eby111 * ebz010, W_110, fma_t(ebx101 * eby110 * ebz011, W_101, fma_t(ebx101 * eby110 * ebz010, W_100, fma_t(ebx100 * eby112 * ebz011, W_021, fma_t(ebx100 * eby112 * ebz010, W_020, fma_t(ebx100 * eby111 * ebz011, W_011, fma_t(ebx100 * eby111 * ebz010, W_010, fma_t(ebx100 * eby110 * ebz011, W_001, ebx100 * eby110 * ebz010 * W_000)))))))))));
      acc[11] += fma_t(ebx101 * eby101 * ebz022, W_112, fma_t(ebx101 * eby101 * ebz021, W_111, fma_t(ebx101 * eby101 * ebz020, W_110, fma_t(ebx101 * eby100 * ebz022, W_102, fma_t(ebx101 * eby100 * ebz021, W_101, fma_t(ebx101 * eby100 * ebz020, W_100, fma_t(ebx100 * eby101 * ebz022, W_012, fma_t(ebx100 * eby101 * ebz021, W_011, fma_t(ebx100 * eby101 * ebz020, W_010, fma_t(ebx100 * eby100 * ebz022, W_002, fma_t(ebx100 * eby100 * ebz021, W_001, ebx100 * eby100 * ebz020 * W_000)))))))))));
      acc[12] += fma_t(ebx123 * ebz101, W_301, fma_t(ebx123 * ebz100, W_300, fma_t(ebx122 * ebz101, W_201, fma_t(ebx122 * ebz100, W_200, fma_t(ebx121 * ebz101, W_101, fma_t(ebx121 * ebz100, W_100, fma_t(ebx120 * ebz101, W_001, ebx120 * ebz100 * W_000)))))));
      acc[13] += fma_t(ebx112 * eby011 * ebz101, W_211, fma_t(ebx112 * eby011 * ebz100, W_210, fma_t(ebx112 * eby010 * ebz101, W_201, fma_t(ebx112 * eby010 * ebz100, W_200, fma_t(ebx111 * eby011 * ebz101, W_111, fma_t(ebx111 * eby011 * ebz100, W_110, fma_t(ebx111 * eby010 * ebz101, W_101, fma_t(ebx111 * eby010 * ebz100, W_100, fma_t(ebx110 * eby011 * ebz101, W_011, fma_t(ebx110 * eby011 * ebz100, W_010, fma_t(ebx110 * eby010 * ebz101, W_001, ebx110 * eby010 * ebz100 * W_000)))))))))));
      acc[14] += fma_t(ebx112 * ebz112, W_202, fma_t(ebx112 * ebz111, W_201, fma_t(ebx112 * ebz110, W_200, fma_t(ebx111 * ebz112, W_102, fma_t(ebx111 * ebz111, W_101, fma_t(ebx111 * ebz110, W_100, fma_t(ebx110 * ebz112, W_002, fma_t(ebx110 * ebz111, W_001, ebx110 * ebz110 * W_000))))))));
      acc[15] += fma_t(ebx101 * eby022 * ebz101, W_121, fma_t(ebx101 * eby022 * ebz100, W_120, fma_t(ebx101 * eby021 * ebz101, W_111, fma_t(ebx101 * eby021 * ebz100, W_110, fma_t(ebx101 * eby020 * ebz101, W_101, fma_t(ebx101 * eby020 * ebz100, W_100, fma_t(ebx100 * eby022 * ebz101, W_021, fma_t(ebx100 * eby022 * ebz100, W_020, fma_t(ebx100 * eby021 * ebz101, W_011, fma_t(ebx100 * eby021 * ebz100, W_010, fma_t(ebx100 * eby020 * ebz101, W_001, ebx100 * eby020 * ebz100 * W_000)))))))))));
      acc[16] += fma_t(ebx101 * eby011 * ebz112, W_112, fma_t(ebx101 * eby011 * ebz111, W_111, fma_t(ebx101 * eby011 * ebz110, W_110, fma_t(ebx101 * eby010 * ebz112, W_102, fma_t(ebx101 * eby010 * ebz111, W_101, fma_t(ebx101 * eby010 * ebz110, W_100, fma_t(ebx100 * eby011 * ebz112, W_012, fma_t(ebx100 * eby011 * ebz111, W_011, fma_t(ebx100 * eby011 * ebz110, W_010, fma_t(ebx100 * eby010 * ebz112, W_002, fma_t(ebx100 * eby010 * ebz111, W_001, ebx100 * eby010 * ebz110 * W_000)))))))))));
      acc[17] += fma_t(ebx101 * ebz123, W_103, fma_t(ebx101 * ebz122, W_102, fma_t(ebx101 * ebz121, W_101, fma_t(ebx101 * ebz120, W_100, fma_t(ebx100 * ebz123, W_003, fma_t(ebx100 * ebz122, W_002, fma_t(ebx100 * ebz121, W_001, ebx100 * ebz120 * W_000)))))));
      acc[18] += fma_t(ebx022 * eby202, W_220, fma_t(ebx022 * eby201, W_210, fma_t(ebx022 * eby200, W_200, fma_t(ebx021 * eby202, W_120, fma_t(ebx021 * eby201, W_110, fma_t(ebx021 * eby200, W_100, fma_t(ebx020 * eby202, W_020, fma_t(ebx020 * eby201, W_010, ebx020 * eby200 * W_000))))))));
      acc[19] += fma_t(ebx011 * eby213, W_130, fma_t(ebx011 * eby212, W_120, fma_t(ebx011 * eby211, W_110, fma_t(ebx011 * eby210, W_100, fma_t(ebx010 * eby213, W_030, fma_t(ebx010 * eby212, W_020, fma_t(ebx010 * eby211, W_010, ebx010 * eby210 * W_000)))))));
      acc[20] += fma_t(ebx011 * eby202 * ebz011, W_121, fma_t(ebx011 * eby202 * ebz010, W_120, fma_t(ebx011 * eby201 * ebz011, W_111, fma_t(ebx011 * eby201 * ebz010, W_110, fma_t(ebx011 * eby200 * ebz011, W_101, fma_t(ebx011 * eby200 * ebz010, W_100, fma_t(ebx010 * eby202 * ebz011, W_021, fma_t(ebx010 * eby202 * ebz010, W_020, fma_t(ebx010 * eby201 * ebz011, W_011, fma_t(ebx010 * eby201 * ebz010, W_010, fma_t(ebx010 * eby200 * ebz011, W_001, ebx010 * eby200 * ebz010 * W_000)))))))))));
      acc[21] += fma_t(eby224, W_040, fma_t(eby223, W_030, fma_t(eby222, W_020, fma_t(eby221, W_010, eby220 * W_000))));
      acc[22] += fma_t(eby213 * ebz011, W_031, fma_t(eby213 * ebz010, W_030, fma_t(eby212 * ebz011, W_021, fma_t(eby212 * ebz010, W_020, fma_t(eby211 * ebz011, W_011, fma_t(eby211 * ebz010, W_010, fma_t(eby210 * ebz011, W_001, eby210 * ebz010 * W_000)))))));
      acc[23] += fma_t(eby202 * ebz022, W_022, fma_t(eby202 * ebz021, W_021, fma_t(eby202 * ebz020, W_020, fma_t(eby201 * ebz022, W_012, fma_t(eby201 * ebz021, W_011, fma_t(eby201 * ebz020, W_010, fma_t(eby200 * ebz022, W_002, fma_t(eby200 * ebz021, W_001, eby200 * ebz020 * W_000))))))));
      acc[24] += fma_t(ebx022 * eby101 * ebz101, W_211, fma_t(ebx022 * eby101 * ebz100, W_210, fma_t(ebx022 * eby100 * ebz101, W_201, fma_t(ebx022 * eby100 * ebz100, W_200, fma_t(ebx021 * eby101 * ebz101, W_111, fma_t(ebx021 * eby101 * ebz100, W_110, fma_t(ebx021 * eby100 * ebz101, W_101, fma_t(ebx021 * eby100 * ebz100, W_100, fma_t(ebx020 * eby101 * ebz101, W_011, fma_t(ebx020 * eby101 * ebz100, W_010, fma_t(ebx020 * eby100 * ebz101, W_001, ebx020 * eby100 * ebz100 * W_000)))))))))));
      acc[25] += fma_t(ebx011 * eby112 * ebz101, W_121, fma_t(ebx011 * eby112 * ebz100, W_120, fma_t(ebx011 * eby111 * ebz101, W_111, fma_t(ebx011 * eby111 * ebz100, W_110, fma_t(ebx011 * eby110 * ebz101, W_101, fma_t(ebx011 * eby110 * ebz100, W_100, fma_t(ebx010 * eby112 * ebz101, W_021, fma_t(ebx010 * eby112 * ebz100, W_020, fma_t(ebx010 * eby111 * ebz101, W_011, fma_t(ebx010 * eby111 * ebz100, W_010, fma_t(ebx010 * eby110 * ebz101, W_001, ebx010 * eby110 * ebz100 * W_000)))))))))));
      acc[26] += fma_t(ebx011 * eby101 * ebz112, W_112, fma_t(ebx011 * eby101 * ebz111, W_111, fma_t(ebx011 * eby101 * ebz110, W_110, fma_t(ebx011 * eby100 * ebz112, W_102, fma_t(ebx011 * eby100 * ebz111, W_101, fma_t(ebx011 * eby100 * ebz110, W_100, fma_t(ebx010 * eby101 * ebz112, W_012, fma_t(ebx010 * eby101 * ebz111, W_011, fma_t(ebx010 * eby101 * ebz110, W_010, fma_t(ebx010 * eby100 * ebz112, W_002, fma_t(ebx010 * eby100 * ebz111, W_001, ebx010 * eby100 * ebz110 * W_000)))))))))));
      acc[27] += fma_t(eby123 * ebz101, W_031, fma_t(eby123 * ebz100, W_030, fma_t(eby122 * ebz101, W_021, fma_t(eby122 * ebz100, W_020, fma_t(eby121 * ebz101, W_011, fma_t(eby121 * ebz100, W_010, fma_t(eby120 * ebz101, W_001, eby120 * ebz100 * W_000)))))));
      acc[28] += fma_t(eby112 * ebz112, W_022, fma_t(eby112 * ebz111, W_021, fma_t(eby112 * ebz110, W_020, fma_t(eby111 * ebz112, W_012, fma_t(eby111 * ebz111, W_011, fma_t(eby111 * ebz110, W_010, fma_t(eby110 * ebz112, W_002, fma_t(eby110 * ebz111, W_001, eby110 * ebz110 * W_000))))))));
      acc[29] += fma_t(eby101 * ebz123, W_013, fma_t(eby101 * ebz122, W_012, fma_t(eby101 * ebz121, W_011, fma_t(eby101 * ebz120, W_010, fma_t(eby100 * ebz123, W_003, fma_t(eby100 * ebz122, W_002, fma_t(eby100 * ebz121, W_001, eby100 * ebz120 * W_000)))))));
      acc[30] += fma_t(ebx022 * ebz202, W_202, fma_t(ebx022 * ebz201, W_201, fma_t(ebx022 * ebz200, W_200, fma_t(ebx021 * ebz202, W_102, fma_t(ebx021 * ebz201, W_101, fma_t(ebx021 * ebz200, W_100, fma_t(ebx020 * ebz202, W_002, fma_t(ebx020 * ebz201, W_001, ebx020 * ebz200 * W_000))))))));
      acc[31] += fma_t(ebx011 * eby011 * ebz202, W_112, fma_t(ebx011 * eby011 * ebz201, W_111, fma_t(ebx011 * eby011 * ebz200, W_110, fma_t(ebx011 * eby010 * ebz202, W_102, fma_t(ebx011 * eby010 * ebz201, W_101, fma_t(ebx011 * eby010 * ebz200, W_100, fma_t(ebx010 * eby011 * ebz202, W_012, fma_t(ebx010 * eby011 * ebz201, W_011, fma_t(ebx010 * eby011 * ebz200, W_010, fma_t(ebx010 * eby010 * ebz202, W_002, fma_t(ebx010 * eby010 * ebz201, W_001, ebx010 * eby010 * ebz200 * W_000)))))))))));
      acc[32] += fma_t(ebx011 * ebz213, W_103, fma_t(ebx011 * ebz212, W_102, fma_t(ebx011 * ebz211, W_101, fma_t(ebx011 * ebz210, W_100, fma_t(ebx010 * ebz213, W_003, fma_t(ebx010 * ebz212, W_002, fma_t(ebx010 * ebz211, W_001, ebx010 * ebz210 * W_000)))))));
      acc[33] += fma_t(eby022 * ebz202, W_022, fma_t(eby022 * ebz201, W_021, fma_t(eby022 * ebz200, W_020, fma_t(eby021 * ebz202, W_012, fma_t(eby021 * ebz201, W_011, fma_t(eby021 * ebz200, W_010, fma_t(eby020 * ebz202, W_002, fma_t(eby020 * ebz201, W_001, eby020 * ebz200 * W_000))))))));
      acc[34] += fma_t(eby011 * ebz213, W_013, fma_t(eby011 * ebz212, W_012, fma_t(eby011 * ebz211, W_011, fma_t(eby011 * ebz210, W_010, fma_t(eby010 * ebz213, W_003, fma_t(eby010 * ebz212, W_002, fma_t(eby010 * ebz211, W_001, eby010 * ebz210 * W_000)))))));
      acc[35] += fma_t(ebz224, W_004, fma_t(ebz223, W_003, fma_t(ebz222, W_002, fma_t(ebz221, W_001, ebz220 * W_000))));
    }
  }
}
