{-# LANGUAGE ForeignFunctionInterface #-}
{-|
Module: Science.QuantumChemistry.GPU
Description: The reference's SCF call surface on one GB300 through libgbhf.

Drop-in replacements, same names and argument meaning, for

  * scfHF          (HartreeFock/HartreeFock.hs:70-87)
  * calcIntegrals  (HartreeFock/HartreeFock.hs:166-181)
  * hcore          (Integrals/IntegralsEvaluation.hs:227-240)
  * mtxOverlap     (Integrals/IntegralsEvaluation.hs:169-177)
  * fock           (HartreeFock/HartreeFock.hs:213-241)
  * energyGradient (HartreeFock/Derivatives.hs:40-48, dead code in the reference)

calling the C ABI of include/gbhf.h (libgbhf.so; link with -lgbhf).  Main.doSCF
(Main.hs:118-125) keeps its code and imports scfHF from here instead of
Science.QuantumChemistry.HartreeFock.HartreeFock.

Status: written against include/gbhf.h but NOT COMPILED in this repository,
whose image has no GHC toolchain.  The struct offsets below are checked
against the C header by tests/test_abi.py.

Contexts: one libgbhf context per process, created on the first call and kept
(device buffers, Boys tables, SAD atoms and tuned task budgets stay resident);
calls take it through an MVar, so they are serialised, as the library requires
per context.  A call on a new context for every SCF costs about 0.14 s instead
of 0.066 s for (H2O)16/6-31G (the bench's e2e_cold_context and e2e).

Basis functions: the direct J/K kernels need each d shell's components in the
order createCGF emits (BasisSet/FetchBasis.hs:50-59: xx, xy, xz, yy, yz, zz);
the sample project "water" "6-31G*" (HsFock/SampleProjects.hs:77-98) lists
xx, yy, zz, xy, xz, yz.  'flatten' reorders the components of each such shell
and every matrix coming back is returned in the caller's own function order.
-}
module Science.QuantumChemistry.GPU
  ( scfHF
  , scfHFWith
  , ScfMode (..)
  , calcIntegrals
  , hcore
  , mtxOverlap
  , fock
  , energyGradient
  , GbhfException (..)
  ) where

import Control.Concurrent.MVar
import Control.Exception (Exception, onException, throwIO)
import Control.Monad (forM_, unless, when)
import Data.Array.Repa (Array, DIM1, U, Z (..), (:.) (..))
import Data.Array.Repa.Repr.Unboxed (fromUnboxed, toUnboxed)
import Data.Int (Int64)
import Data.List (sortBy)
import qualified Data.Map as M
import Data.Ord (comparing)
import qualified Data.Vector.Storable as VS
import qualified Data.Vector.Storable.Mutable as VSM
import qualified Data.Vector.Unboxed as VU
import Foreign
import Foreign.C.String (CString, peekCString)
import Foreign.C.Types
import System.IO.Unsafe (unsafePerformIO)
import Text.Printf (printf)

import Science.QuantumChemistry.GlobalTypes
import Science.QuantumChemistry.NumericalTools.TableBoys (Boys)

-- ----------------------------------------------------------- C ABI ----

data GbhfCtx

type Status = CInt

foreign import ccall safe "gbhf_create"
  c_gbhf_create :: Ptr (Ptr GbhfCtx) -> CInt -> IO Status
foreign import ccall safe "gbhf_destroy"
  c_gbhf_destroy :: Ptr GbhfCtx -> IO Status
foreign import ccall safe "gbhf_last_error"
  c_gbhf_last_error :: Ptr GbhfCtx -> IO CString
foreign import ccall safe "gbhf_set_basis"
  c_gbhf_set_basis :: Ptr GbhfCtx -> CInt -> Ptr CDouble -> Ptr CDouble -> CInt -> Ptr CInt -> Ptr CInt
                   -> Ptr CInt -> Ptr CDouble -> Ptr CDouble -> IO Status
foreign import ccall safe "gbhf_set_boys_grid"
  c_gbhf_set_boys_grid :: Ptr GbhfCtx -> Ptr CDouble -> IO Status
foreign import ccall safe "gbhf_generate_boys_grid"
  c_gbhf_generate_boys_grid :: Ptr GbhfCtx -> Ptr CDouble -> IO Status
foreign import ccall safe "gbhf_overlap"
  c_gbhf_overlap :: Ptr GbhfCtx -> CInt -> Ptr CDouble -> IO Status
foreign import ccall safe "gbhf_hcore"
  c_gbhf_hcore :: Ptr GbhfCtx -> CInt -> Ptr CDouble -> IO Status
foreign import ccall unsafe "gbhf_eri_canonical_length"
  c_gbhf_eri_canonical_length :: CInt -> Int64
foreign import ccall safe "gbhf_eri_canonical"
  c_gbhf_eri_canonical :: Ptr GbhfCtx -> CInt -> Ptr CDouble -> Int64 -> IO Status
foreign import ccall safe "gbhf_fock"
  c_gbhf_fock :: Ptr GbhfCtx -> CInt -> CInt -> CDouble -> CDouble -> Ptr CDouble -> Ptr CDouble
              -> Ptr CDouble -> IO Status
foreign import ccall safe "gbhf_scf_opts_reference"
  c_gbhf_scf_opts_reference :: Ptr ScfOpts -> IO ()
foreign import ccall safe "gbhf_scf_opts_baseline"
  c_gbhf_scf_opts_baseline :: Ptr ScfOpts -> IO ()
foreign import ccall safe "gbhf_scf"
  c_gbhf_scf :: Ptr GbhfCtx -> Ptr ScfOpts -> Ptr ScfResult -> IO Status
foreign import ccall safe "gbhf_scf_trace"
  c_gbhf_scf_trace :: Ptr GbhfCtx -> Ptr CDouble -> CInt -> Ptr CInt -> IO Status
foreign import ccall safe "gbhf_gradient"
  c_gbhf_gradient :: Ptr GbhfCtx -> CInt -> CDouble -> Ptr CDouble -> Ptr CDouble -> Ptr CDouble -> IO Status

-- gbhf_mode, gbhf_precision, gbhf_guess (include/gbhf.h)
modeReference, modeExact, precFP64, precMixed, guessSAD :: CInt
modeReference = 0
modeExact = 1
precFP64 = 0
precMixed = 1
guessSAD = 2

-- | gbhf_scf_opts: 9 ints, 8 doubles from offset 40, autotune at 104; 112 bytes.
data ScfOpts = ScfOpts
  { oMode, oPrecision, oGuess, oDiisSize, oMaxIter, oIncremental, oFullRebuildEvery, oFinalFP64
  , oRefStopRule :: !CInt
  , oConvError, oConvEnergy, oConvDensity, oDiisStart, oSchwarz, oMixedCutoff, oCharge
  , oGradMixedCutoff :: !CDouble
  , oAutotune :: !CInt
  }

scfOptsIntOffsets :: [Int]
scfOptsIntOffsets = [0, 4, 8, 12, 16, 20, 24, 28, 32]

scfOptsDoubleOffsets :: [Int]
scfOptsDoubleOffsets = [40, 48, 56, 64, 72, 80, 88, 96]

scfOptsAutotuneOffset, scfOptsSize :: Int
scfOptsAutotuneOffset = 104
scfOptsSize = 112

instance Storable ScfOpts where
  sizeOf _ = scfOptsSize
  alignment _ = 8
  peek p = do
    [a, b, c, d, e, f, g, h, i] <- mapM (peekByteOff p) scfOptsIntOffsets
    [j, k, l, m, n, o, q, r] <- mapM (peekByteOff p) scfOptsDoubleOffsets
    s <- peekByteOff p scfOptsAutotuneOffset
    return (ScfOpts a b c d e f g h i j k l m n o q r s)
  poke p x = do
    zipWithM_' (pokeByteOff p) scfOptsIntOffsets
      [ oMode x, oPrecision x, oGuess x, oDiisSize x, oMaxIter x, oIncremental x, oFullRebuildEvery x
      , oFinalFP64 x, oRefStopRule x ]
    zipWithM_' (pokeByteOff p) scfOptsDoubleOffsets
      [ oConvError x, oConvEnergy x, oConvDensity x, oDiisStart x, oSchwarz x, oMixedCutoff x, oCharge x
      , oGradMixedCutoff x ]
    pokeByteOff p scfOptsAutotuneOffset (oAutotune x)

zipWithM_' :: (a -> b -> IO ()) -> [a] -> [b] -> IO ()
zipWithM_' f xs ys = sequence_ (zipWith f xs ys)

-- | gbhf_result: energy 0, iterations 8, converged 12, n_occupied 16,
-- nuclear_repulsion 24, fock_flat 32, coeff 40, density_flat 48,
-- orb_energies 56, statistics 64..96; 104 bytes.
data ScfResult

scfResultSize :: Int
scfResultSize = 104

resEnergy, resIterations, resConverged, resNOccupied, resFock, resCoeff, resDensity, resOrbE :: Int
resEnergy = 0
resIterations = 8
resConverged = 12
resNOccupied = 16
resFock = 32
resCoeff = 40
resDensity = 48
resOrbE = 56

-- ------------------------------------------------------ errors ----

-- | A libgbhf status other than GBHF_OK with its message.  Status 2
-- (GBHF_ERR_NOT_CONVERGED) is the reference's error "SCF maxium steps
-- exceeded" (HartreeFock.hs:123); 8 (GBHF_ERR_INDEX) its out-of-bounds Harris
-- lookup (HartreeFock.hs:143-146); 1 (GBHF_ERR_BAD_INPUT) HSFOCKException.
data GbhfException = GbhfException Int String deriving Show
instance Exception GbhfException

check :: Ptr GbhfCtx -> String -> Status -> IO ()
check ctx what st = unless (st == 0) $ do
  msg <- c_gbhf_last_error ctx >>= peekCString
  if st == 2
    then error "SCF maxium steps exceeded"
    else throwIO (GbhfException (fromIntegral st) (what ++ ": " ++ msg))

-- ----------------------------------------------------- context ----

{-# NOINLINE sharedContext #-}
sharedContext :: MVar (Ptr GbhfCtx)
sharedContext = unsafePerformIO newEmptyMVar

-- | Run with the process's context (device 0), creating it on first use;
-- calls are serialised on it.
withContext :: (Ptr GbhfCtx -> IO a) -> IO a
withContext act = do
  mctx <- tryTakeMVar sharedContext
  ctx <- case mctx of
    Just c -> return c
    Nothing -> alloca $ \pp -> do
      st <- c_gbhf_create pp 0
      unless (st == 0) $ throwIO (GbhfException (fromIntegral st) "gbhf_create: no usable GPU")
      peek pp
  r <- act ctx `onException` putMVar sharedContext ctx
  putMVar sharedContext ctx
  return r

-- ------------------------------------------------------- basis ----

-- | Cartesian exponents of a function type (mapLAngular, GlobalTypes.hs:263-284).
lxyz :: Funtype -> [Int]
lxyz ft = [M.findWithDefault 0 (ft, k) mapLAngular | k <- [0, 1, 2]]

-- | createCGF's order of the d components (FetchBasis.hs:50-59).
dRank :: Funtype -> Int
dRank ft = case ft of
  Dxx -> 0
  Dxy -> 1
  Dxz -> 2
  Dyy -> 3
  Dyz -> 4
  Dzz -> 5
  _ -> -1

-- | [AtomData] in structure-of-arrays form, CGFs in the order the kernels need,
-- with perm !! k = the caller's index of function k.
data Flat = Flat
  { fAtoms :: Int, fXYZ :: [Double], fZ :: [Double], fNCgf :: Int, fCgfAtom :: [Int], fLxyz :: [Int]
  , fNPrim :: [Int], fCoef :: [Double], fExpo :: [Double], fPerm :: [Int] }

flatten :: [AtomData] -> Flat
flatten atoms = Flat
  { fAtoms = length atoms
  , fXYZ = concatMap getCoord atoms
  , fZ = map getZnumber atoms
  , fNCgf = length cgfs
  , fCgfAtom = map (\(a, _, _) -> a) cgfs
  , fLxyz = concatMap (\(_, _, CGF _ ft) -> lxyz ft) cgfs
  , fNPrim = map (\(_, _, CGF ps _) -> length ps) cgfs
  , fCoef = concatMap (\(_, _, CGF ps _) -> map fst ps) cgfs
  , fExpo = concatMap (\(_, _, CGF ps _) -> map snd ps) cgfs
  , fPerm = map (\(_, k, _) -> k) cgfs
  }
  where
    numbered = zip [0 :: Int ..] [(ia, cgf) | (ia, at) <- zip [0 ..] atoms, cgf <- getBasis at]
    cgfs = concatMap reorder (runs numbered)
    -- consecutive d functions of one atom with the same exponents, each
    -- component at most once, form one shell
    runs [] = []
    runs (x@(_, (ia, CGF ps ft)) : rest)
      | dRank ft >= 0 = let (grp, others) = shell [dRank ft] rest in (x : grp) : runs others
      | otherwise = [x] : runs rest
      where
        shell seen (y@(_, (ib, CGF qs gt)) : more)
          | ib == ia && dRank gt >= 0 && dRank gt `notElem` seen && map snd qs == map snd ps =
              let (g, o) = shell (dRank gt : seen) more in (y : g, o)
        shell _ more = ([], more)
    reorder grp = [(ia, k, cgf) | (k, (ia, cgf)) <- sortBy (comparing (\(_, (_, CGF _ ft)) -> dRank ft)) grp]

upload :: Ptr GbhfCtx -> Flat -> IO ()
upload ctx f =
  withArray (map realToFrac (fXYZ f)) $ \pxyz ->
  withArray (map realToFrac (fZ f)) $ \pz ->
  withArray (map fromIntegral (fCgfAtom f)) $ \pa ->
  withArray (map fromIntegral (fLxyz f)) $ \pl ->
  withArray (map fromIntegral (fNPrim f)) $ \pn ->
  withArray (map realToFrac (fCoef f)) $ \pc ->
  withArray (map realToFrac (fExpo f)) $ \pe ->
    c_gbhf_set_basis ctx (fromIntegral (fAtoms f)) pxyz pz (fromIntegral (fNCgf f)) pa pl pn pc pe
      >>= check ctx "gbhf_set_basis"

-- | Index of (i, j), i <= j, in the flat upper triangle (indexDIM2toFlat,
-- NumericalTools/LinearAlgebra.hs:250-253).
flatIndex :: Int -> Int -> Int -> Int
flatIndex n i j = let (a, b) = (min i j, max i j) in a * n - (a * (a - 1)) `div` 2 + (b - a)

-- | A flat matrix in kernel order back in the caller's function order.
unpermuteFlat :: [Int] -> VU.Vector Double -> VU.Vector Double
unpermuteFlat perm v
  | perm == [0 .. n - 1] = v
  | otherwise = VU.generate (VU.length v) pick
  where
    n = length perm
    inv = VU.update (VU.replicate n 0) (VU.fromList (zip perm [0 ..]))
    rows = VU.fromList [(i, j) | i <- [0 .. n - 1], j <- [i .. n - 1]]
    pick t = let (i, j) = rows VU.! t in v VU.! flatIndex n (inv VU.! i) (inv VU.! j)

-- | Rows of an N x N matrix (coefficients: functions x orbitals) back in the caller's order.
unpermuteRows :: [Int] -> VU.Vector Double -> VU.Vector Double
unpermuteRows perm v
  | perm == [0 .. n - 1] = v
  | otherwise = VU.generate (n * n) (\t -> let (i, c) = t `divMod` n in v VU.! ((inv VU.! i) * n + c))
  where
    n = length perm
    inv = VU.update (VU.replicate n 0) (VU.fromList (zip perm [0 ..]))

-- | A flat matrix in the caller's order into kernel order.
permuteFlat :: [Int] -> VU.Vector Double -> VU.Vector Double
permuteFlat perm v
  | perm == [0 .. n - 1] = v
  | otherwise = VU.fromList [v VU.! flatIndex n (p VU.! i) (p VU.! j) | i <- [0 .. n - 1], j <- [i .. n - 1]]
  where
    n = length perm
    p = VU.fromList perm

toC :: VU.Vector Double -> VS.Vector CDouble
toC = VS.fromList . map realToFrac . VU.toList

fromC :: VS.Vector CDouble -> VU.Vector Double
fromC = VU.fromList . map realToFrac . VS.toList

-- Output buffer of n doubles filled by `fill`.
buffer :: Int -> (Ptr CDouble -> IO ()) -> IO (VU.Vector Double)
buffer n fill = do
  mv <- VSM.new n
  VSM.unsafeWith mv fill
  fromC <$> VS.freeze mv

-- ----------------------------------------------------- the API ----

-- | Numerics and driver: the reference's own (tabulated Boys grid, primitive
-- screening, stored ERIs, Harris guess, DIIS 5, 30 steps, stop at max|e| <
-- 1e-7), or direct J/K in FP64 or mixed FP32/FP64 (SAD start, DIIS 6, stop at
-- |dE| < 1e-10 and RMS dD < 1e-8).
data ScfMode = Reference | ExactFP64 | ExactMixed deriving (Eq, Show)

-- | scfHF :: [AtomData] -> Charge -> (String -> IO ()) -> IO HFData (HartreeFock.hs:70)
scfHF :: [AtomData] -> Charge -> (String -> IO ()) -> IO HFData
scfHF = scfHFWith Reference

scfHFWith :: ScfMode -> [AtomData] -> Charge -> (String -> IO ()) -> IO HFData
scfHFWith mode atoms charge logger = withContext $ \ctx -> do
  let f = flatten atoms
      n = fNCgf f
      ntri = n * (n + 1) `div` 2
  upload ctx f
  when (mode == Reference) $ c_gbhf_generate_boys_grid ctx nullPtr >>= check ctx "gbhf_generate_boys_grid"
  opts <- alloca $ \po -> do
    (if mode == Reference then c_gbhf_scf_opts_reference else c_gbhf_scf_opts_baseline) po
    o <- peek po
    return o { oCharge = realToFrac charge
             , oPrecision = if mode == ExactMixed then precMixed else precFP64
             , oIncremental = if mode == ExactMixed then 1 else 0
             , oGuess = if mode == Reference then oGuess o else guessSAD }
  fockV <- VSM.new ntri
  coeffV <- VSM.new (n * n)
  densV <- VSM.new ntri
  orbV <- VSM.new n
  energy <-
    VSM.unsafeWith fockV $ \pf -> VSM.unsafeWith coeffV $ \pc -> VSM.unsafeWith densV $ \pd ->
    VSM.unsafeWith orbV $ \pe -> with opts $ \po -> allocaBytesAligned scfResultSize 8 $ \pr -> do
      fillBytes pr 0 scfResultSize
      pokeByteOff pr resFock pf
      pokeByteOff pr resCoeff pc
      pokeByteOff pr resDensity pd
      pokeByteOff pr resOrbE pe
      st <- c_gbhf_scf ctx po (castPtr pr)
      logTrace ctx logger
      check ctx "gbhf_scf" st
      realToFrac <$> (peekByteOff pr resEnergy :: IO CDouble)
  fockF <- fromC <$> VS.freeze fockV
  coeffF <- fromC <$> VS.freeze coeffV
  densF <- fromC <$> VS.freeze densV
  orbF <- fromC <$> VS.freeze orbV
  let perm = fPerm f
  logger (printf "HF energy %.10f\n" energy)
  return HFData
    { getFock = fromUnboxed (Z :. ntri) (unpermuteFlat perm fockF)
    , getCoeff = fromUnboxed (Z :. n :. n) (unpermuteRows perm coeffF)
    , getDensity = fromUnboxed (Z :. ntri) (unpermuteFlat perm densF)
    , getOrbE = orbF
    , getEnergy = energy
    }

-- | One line per SCF step (gbhf_scf_trace) instead of the reference's show
-- dumps of its matrices (HartreeFock.hs:116-117).
logTrace :: Ptr GbhfCtx -> (String -> IO ()) -> IO ()
logTrace ctx logger = alloca $ \pn -> do
  _ <- c_gbhf_scf_trace ctx nullPtr 0 pn
  nrec <- fromIntegral <$> peek pn
  recs <- buffer (max 1 nrec * 8) (\p -> () <$ c_gbhf_scf_trace ctx p (fromIntegral nrec) pn)
  forM_ [0 .. nrec - 1] $ \k ->
    logger (printf "step %d: E = %.10f  dE = %.3e  rms dD = %.3e  max|e| = %.3e\n"
              (round (recs VU.! (8 * k)) :: Int) (recs VU.! (8 * k + 1)) (recs VU.! (8 * k + 2))
              (recs VU.! (8 * k + 3)) (recs VU.! (8 * k + 4)))

-- | calcIntegrals :: Map Boys Double -> [AtomData] -> Array U DIM1 Double
-- (HartreeFock.hs:166-181): the caller's Boys grid (15 x 1001 values of
-- generateGridBoys 0.1, in key order) goes to the device, which evaluates
-- every canonical ERI with the reference's numerics.
calcIntegrals :: M.Map Boys Double -> [AtomData] -> Array U DIM1 Double
calcIntegrals grid atoms = unsafePerformIO $ withContext $ \ctx -> do
  let f = flatten atoms
      n = fNCgf f
      len = c_gbhf_eri_canonical_length (fromIntegral n)
  unless (fPerm f == [0 .. n - 1]) $
    throwIO (GbhfException 7 "calcIntegrals: d components outside createCGF order")
  upload ctx f
  setGrid ctx grid
  v <- buffer (fromIntegral len) (\p -> c_gbhf_eri_canonical ctx modeReference p len >>= check ctx "gbhf_eri_canonical")
  return (fromUnboxed (Z :. fromIntegral len) v)

setGrid :: Ptr GbhfCtx -> M.Map Boys Double -> IO ()
setGrid ctx grid
  | M.size grid == 15 * 1001 =
      VS.unsafeWith (VS.fromList (map realToFrac (M.elems grid))) $ \p ->
        c_gbhf_set_boys_grid ctx p >>= check ctx "gbhf_set_boys_grid"
  | otherwise = c_gbhf_generate_boys_grid ctx nullPtr >>= check ctx "gbhf_generate_boys_grid"

oneElectron :: (Ptr GbhfCtx -> CInt -> Ptr CDouble -> IO Status) -> String -> Maybe (M.Map Boys Double)
            -> [AtomData] -> IO (Array U DIM1 Double)
oneElectron call what grid atoms = withContext $ \ctx -> do
  let f = flatten atoms
      n = fNCgf f
      ntri = n * (n + 1) `div` 2
  upload ctx f
  maybe (return ()) (setGrid ctx) grid
  v <- buffer ntri (\p -> call ctx modeReference p >>= check ctx what)
  return (fromUnboxed (Z :. ntri) (unpermuteFlat (fPerm f) v))

-- | hcore :: Monad m => Map Boys Double -> [AtomData] -> m (Array U DIM1 Double)
hcore :: M.Map Boys Double -> [AtomData] -> IO (Array U DIM1 Double)
hcore grid = oneElectron c_gbhf_hcore "gbhf_hcore" (Just grid)

-- | mtxOverlap :: Monad m => [AtomData] -> m (Array U DIM1 Double)
mtxOverlap :: [AtomData] -> IO (Array U DIM1 Double)
mtxOverlap = oneElectron c_gbhf_overlap "gbhf_overlap" Nothing

-- | fock :: Monad m => [AtomData] -> FlattenCore -> FlattenChargeDensity -> Integrals -> m (Array U DIM1 Double)
-- (HartreeFock.hs:213): F = H + G(D) by the direct J/K build in FP64 (the
-- stored integrals are not needed; exact numerics, Schwarz cutoff 1e-12).
fock :: [AtomData] -> FlattenCore -> FlattenChargeDensity -> Integrals -> IO (Array U DIM1 Double)
fock atoms core dens _ = withContext $ \ctx -> do
  let f = flatten atoms
      n = fNCgf f
      ntri = n * (n + 1) `div` 2
      perm = fPerm f
  upload ctx f
  v <- VS.unsafeWith (toC (permuteFlat perm (toUnboxed core))) $ \ph ->
       VS.unsafeWith (toC (permuteFlat perm (toUnboxed dens))) $ \pd ->
       buffer ntri (\pf -> c_gbhf_fock ctx modeExact precFP64 1e-12 1e-4 ph pd pf >>= check ctx "gbhf_fock")
  return (fromUnboxed (Z :. ntri) (unpermuteFlat perm v))

-- | energyGradient :: Monad m => [AtomData] -> HFData -> m Gradient
-- (Derivatives.hs:40): dE/dR from the density D of the HFData and the
-- energy-weighted density W = 2 sum_occ eps_i C_i C_i^T, which for a
-- converged SCF equals D F D / 2 (F C = S C eps, D = 2 C_occ C_occ^T);
-- hartree/bohr, 3 per atom.
energyGradient :: [AtomData] -> HFData -> IO Gradient
energyGradient atoms hf = withContext $ \ctx -> do
  let f = flatten atoms
      n = fNCgf f
      natoms = fAtoms f
      perm = fPerm f
      dflat = toUnboxed (getDensity hf)
      d = square n dflat
      fk = square n (toUnboxed (getFock hf))
      dfd = matmul n (matmul n d fk) d
      w = VU.fromList [0.5 * dfd VU.! (i * n + j) | i <- [0 .. n - 1], j <- [i .. n - 1]]
  upload ctx f
  g <- VS.unsafeWith (toC (permuteFlat perm dflat)) $ \pd ->
       VS.unsafeWith (toC (permuteFlat perm w)) $ \pw ->
       buffer (3 * natoms) (\pg -> c_gbhf_gradient ctx precFP64 1e-12 pd pw pg >>= check ctx "gbhf_gradient")
  return (fromUnboxed (Z :. 3 * natoms) g)

-- | N x N row-major matrix of a flat upper triangle.
square :: Int -> VU.Vector Double -> VU.Vector Double
square n v = VU.generate (n * n) (\t -> let (i, j) = t `divMod` n in v VU.! flatIndex n i j)

matmul :: Int -> VU.Vector Double -> VU.Vector Double -> VU.Vector Double
matmul n a b = VU.generate (n * n) (\t -> let (i, j) = t `divMod` n
                                          in sum [a VU.! (i * n + k) * b VU.! (k * n + j) | k <- [0 .. n - 1]])
