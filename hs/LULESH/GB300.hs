{-# LANGUAGE BangPatterns             #-}
{-# LANGUAGE ForeignFunctionInterface #-}
-- |
-- Module      : LULESH.GB300
--
-- The LULESH step of src/LULESH.hs (@lulesh@ :37-53, @lagrangeLeapFrog@
-- :66-102, @timeIncrement@ :1166-1213) on a GB300, through the C ABI of
-- liblulesh_gb300.so (include/lulesh_gb300.h).
--
-- It binds C the way the reference already does for its output path
-- (src/VisIt.hs:71-86 -> cbits/visit.cc:149-177): @foreign import ccall@ with
-- one @Ptr R@ per structure-of-arrays component of the 'Domain', taken with
-- @ptrsOfArrayData@ and kept alive with @touchArrayData@ (src/VisIt.hs:43-68).
-- Calls are @safe@: they may block on the GPU, and the executable is already
-- built @-threaded@ (lulesh-accelerate.cabal:54).
--
-- Drop-in use in src/Main.hs: 'simulateGB300' replaces @simulate@ (:90-108),
-- whose step is @$( PTX.runQ lulesh ) mN0 v0@; the context computes the nodal
-- mass and reference volume (@mN0@, @v0@) of the same cube itself.  The
-- library follows the C reference (reference/C/LULESH-OMP.cc) where the
-- Haskell port differs, so its results are LULESH-OMP's.
--
-- This module is not compiled by this repository's build (there is no GHC
-- toolchain here); tests/test_haskell_binding.py checks every foreign import
-- below, name and arity, against include/lulesh_gb300.h.
module LULESH.GB300
  ( Context
  , LuleshException(..)
  , withContext
  , uploadDomain
  , downloadDomain
  , stepGB300
  , runGB300
  , simulateGB300
  , originEnergy
  , symmetryCheck
  ) where

import Domain
import Type

import Data.Array.Accelerate                            ( Array(..), Z(..), (:.)(..), indexArray )
import Data.Array.Accelerate.Array.Data                 ( ptrsOfArrayData, touchArrayData )
import Data.Array.Accelerate.Array.Sugar                ( allocateArray )

import Control.Exception                                ( Exception, bracket, throwIO )
import Control.Monad                                    ( when )
import Foreign.C.String                                 ( CString, peekCString )
import Foreign.C.Types                                  ( CInt(..), CLong(..) )
import Foreign.Marshal.Alloc                            ( alloca )
import Foreign.Ptr                                      ( Ptr, nullPtr )
import Foreign.Storable                                 ( peek )


-- | An opaque lulesh_ctx: the device state of one problem, its stream and
-- its captured run-loop graph.
data LuleshCtx
newtype Context = Context (Ptr LuleshCtx)

-- | The reference's exit codes (LULESH-OMP.cc:82) and the library's own.
data LuleshException
  = VolumeError String          -- ^ -1
  | QStopError String           -- ^ -2
  | CudaError String            -- ^ -3
  | RunTimeout String           -- ^ -4: a run stopped short of stoptime
  | BadArgument String          -- ^ -5
  | OtherError Int String
  deriving Show

instance Exception LuleshException


-- Foreign imports (include/lulesh_gb300.h) ----------------------------------

foreign import ccall safe "lulesh_create"
  c_lulesh_create :: CInt -> CInt -> CInt -> Ptr () -> Ptr (Ptr LuleshCtx) -> IO CInt

foreign import ccall safe "lulesh_destroy"
  c_lulesh_destroy :: Ptr LuleshCtx -> IO ()

foreign import ccall safe "lulesh_last_error"
  c_lulesh_last_error :: Ptr LuleshCtx -> IO CString

foreign import ccall safe "lulesh_sizes"
  c_lulesh_sizes :: Ptr LuleshCtx -> Ptr CInt -> Ptr CLong -> Ptr CLong -> IO CInt

foreign import ccall safe "lulesh_time_increment"
  c_lulesh_time_increment :: Ptr LuleshCtx -> IO CInt

foreign import ccall safe "lulesh_lagrange_nodal"
  c_lulesh_lagrange_nodal :: Ptr LuleshCtx -> IO CInt

foreign import ccall safe "lulesh_lagrange_elements"
  c_lulesh_lagrange_elements :: Ptr LuleshCtx -> IO CInt

foreign import ccall safe "lulesh_calc_time_constraints"
  c_lulesh_calc_time_constraints :: Ptr LuleshCtx -> IO CInt

foreign import ccall safe "lulesh_lagrange_leapfrog"
  c_lulesh_lagrange_leapfrog :: Ptr LuleshCtx -> IO CInt

foreign import ccall safe "lulesh_run"
  c_lulesh_run :: Ptr LuleshCtx -> CInt -> Ptr CInt -> IO CInt

foreign import ccall safe "lulesh_upload_domain"
  c_lulesh_upload_domain
    :: Ptr LuleshCtx
    -> Ptr R -> Ptr R -> Ptr R          -- x y z
    -> Ptr R -> Ptr R -> Ptr R          -- xd yd zd
    -> Ptr R -> Ptr R -> Ptr R          -- e p q
    -> Ptr R -> Ptr R                   -- v ss
    -> R -> R                           -- time deltatime
    -> IO CInt

foreign import ccall safe "lulesh_download_domain"
  c_lulesh_download_domain
    :: Ptr LuleshCtx
    -> Ptr R -> Ptr R -> Ptr R
    -> Ptr R -> Ptr R -> Ptr R
    -> Ptr R -> Ptr R -> Ptr R
    -> Ptr R -> Ptr R
    -> Ptr R -> Ptr R                   -- time deltatime (out)
    -> IO CInt

foreign import ccall safe "lulesh_origin_energy"
  c_lulesh_origin_energy :: Ptr LuleshCtx -> Ptr R -> IO CInt

foreign import ccall safe "lulesh_symmetry"
  c_lulesh_symmetry :: Ptr LuleshCtx -> Ptr R -> Ptr R -> Ptr R -> IO CInt


-- Contexts -------------------------------------------------------------------

-- | LULESH 1.0 initial conditions, as src/Main.hs:60-83 sets them up
-- (e = 3.948746e7 in the origin element, dt0 = 1e-7).
initV1 :: CInt
initV1 = 1

precisionFP64 :: CInt
precisionFP64 = 0

check :: Context -> CInt -> IO ()
check (Context p) rc
  | rc == 0   = return ()
  | otherwise = do
      msg <- peekCString =<< c_lulesh_last_error p
      throwIO $ case rc of
        -1 -> VolumeError msg
        -2 -> QStopError msg
        -3 -> CudaError msg
        -4 -> RunTimeout msg
        -5 -> BadArgument msg
        _  -> OtherError (fromIntegral rc) msg

-- | A context for the numElem^3 Sedov problem on the current CUDA device,
-- in plain FP64 (the drop-in precision), destroyed when the action ends.
withContext :: Int -> (Context -> IO a) -> IO a
withContext numElem = bracket create destroy
  where
    create = alloca $ \pp -> do
      rc <- c_lulesh_create (fromIntegral numElem) initV1 precisionFP64 nullPtr pp
      when (rc /= 0) $ do
        msg <- peekCString =<< c_lulesh_last_error nullPtr
        throwIO (BadArgument msg)
      Context <$> peek pp
    destroy (Context p) = c_lulesh_destroy p


-- The Domain record across the FFI --------------------------------------------

-- | Copy a 'Domain' (src/Domain.hs:11-21) into the context's device state.
uploadDomain :: Context -> Domain -> IO ()
uploadDomain ctx@(Context p) (Array _ ad_pos, Array _ ad_vel, Array _ ad_e, Array _ ad_p, Array _ ad_q,
                              Array _ ad_v, Array _ ad_ss, t, dt) = do
  let ((((), p_x),  p_y),  p_z)  = ptrsOfArrayData ad_pos
      ((((), p_xd), p_yd), p_zd) = ptrsOfArrayData ad_vel
  rc <- c_lulesh_upload_domain p p_x p_y p_z p_xd p_yd p_zd
          (ptrsOfArrayData ad_e) (ptrsOfArrayData ad_p) (ptrsOfArrayData ad_q)
          (ptrsOfArrayData ad_v) (ptrsOfArrayData ad_ss)
          (t `indexArray` Z) (dt `indexArray` Z)
  touchArrayData ad_pos
  touchArrayData ad_vel
  touchArrayData ad_e
  touchArrayData ad_p
  touchArrayData ad_q
  touchArrayData ad_v
  touchArrayData ad_ss
  check ctx rc

-- | A fresh 'Domain' holding the context's current state.
downloadDomain :: Context -> IO Domain
downloadDomain ctx@(Context p) = do
  (ne, nn) <- edges ctx
  pos@(Array _ ad_pos) <- allocateArray (Z :. nn :. nn :. nn)
  vel@(Array _ ad_vel) <- allocateArray (Z :. nn :. nn :. nn)
  fe@(Array _ ad_e)    <- allocateArray (Z :. ne :. ne :. ne)
  fp@(Array _ ad_p)    <- allocateArray (Z :. ne :. ne :. ne)
  fq@(Array _ ad_q)    <- allocateArray (Z :. ne :. ne :. ne)
  fv@(Array _ ad_v)    <- allocateArray (Z :. ne :. ne :. ne)
  fss@(Array _ ad_ss)  <- allocateArray (Z :. ne :. ne :. ne)
  t@(Array _ ad_t)     <- allocateArray Z
  dt@(Array _ ad_dt)   <- allocateArray Z
  let ((((), p_x),  p_y),  p_z)  = ptrsOfArrayData ad_pos
      ((((), p_xd), p_yd), p_zd) = ptrsOfArrayData ad_vel
  rc <- c_lulesh_download_domain p p_x p_y p_z p_xd p_yd p_zd
          (ptrsOfArrayData ad_e) (ptrsOfArrayData ad_p) (ptrsOfArrayData ad_q)
          (ptrsOfArrayData ad_v) (ptrsOfArrayData ad_ss)
          (ptrsOfArrayData ad_t) (ptrsOfArrayData ad_dt)
  mapM_ touchArrayData [ad_e, ad_p, ad_q, ad_v, ad_ss, ad_t, ad_dt]
  touchArrayData ad_pos
  touchArrayData ad_vel
  check ctx rc
  return (pos, vel, fe, fp, fq, fv, fss, t, dt)

edges :: Context -> IO (Int, Int)
edges ctx@(Context p) =
  alloca $ \ps -> alloca $ \pe -> alloca $ \pn -> do
    check ctx =<< c_lulesh_sizes p ps pe pn
    s <- fromIntegral <$> peek ps
    return (s, s + 1)


-- The step -------------------------------------------------------------------

-- | One cycle, as @$( PTX.runQ lulesh ) mN0 v0@ in src/Main.hs:99-108:
-- TimeIncrement then LagrangeLeapFrog (LULESH-OMP.cc:3184-3185), on the state
-- the 'Domain' holds.  The state crosses the FFI both ways; a loop that keeps
-- it on the device uses 'runGB300' or the per-cycle calls directly.
stepGB300 :: Context -> Domain -> IO Domain
stepGB300 ctx@(Context p) dom = do
  uploadDomain ctx dom
  check ctx =<< c_lulesh_time_increment p
  check ctx =<< c_lulesh_lagrange_leapfrog p
  downloadDomain ctx

-- | Up to maxSteps cycles of the reference main loop (LULESH-OMP.cc:3179-3188)
-- on the device, in one CUDA graph launch; returns the cycles done.
runGB300 :: Context -> Int -> IO Int
runGB300 ctx@(Context p) maxSteps =
  alloca $ \pn -> do
    check ctx =<< c_lulesh_run p (fromIntegral maxSteps) pn
    fromIntegral <$> peek pn

-- | The replacement for @simulate@ (src/Main.hs:90-108): the state goes to
-- the device once and stays there.  Without a writer the whole loop runs on
-- the device ('runGB300'); with one (the @--output@ path of src/Main.hs:85-88)
-- each cycle's starting state is downloaded and written first, as @simulate@
-- writes it.
simulateGB300 :: Context -> Int -> Maybe (Int -> Domain -> IO ()) -> Domain -> IO (Domain, Int)
simulateGB300 ctx@(Context p) maxSteps writer dom0 = do
  uploadDomain ctx dom0
  n <- case writer of
         Nothing    -> runGB300 ctx maxSteps
         Just write -> loop write 0
  dom <- downloadDomain ctx
  return (dom, n)
  where
    loop write !i
      | i >= maxSteps = return i
      | otherwise     = do
          dom@(_, _, _, _, _, _, _, t, _) <- downloadDomain ctx
          if t `indexArray` Z >= t_end parameters
            then return i
            else do
              write i dom
              check ctx =<< c_lulesh_time_increment p
              check ctx =<< c_lulesh_lagrange_leapfrog p
              loop write (i + 1)


-- Result checks ----------------------------------------------------------------

-- | Energy of the origin element (the reference's "Final Origin Energy").
originEnergy :: Context -> IO R
originEnergy ctx@(Context p) =
  alloca $ \pe -> do
    check ctx =<< c_lulesh_origin_energy p pe
    peek pe

-- | The plane-0 symmetry test of LULESH-OMP.cc:3197-3223 / src/Main.hs:132-156:
-- (maximum absolute, total absolute, maximum relative difference).
symmetryCheck :: Context -> IO (R, R, R)
symmetryCheck ctx@(Context p) =
  alloca $ \pa -> alloca $ \pt -> alloca $ \pr -> do
    check ctx =<< c_lulesh_symmetry p pa pt pr
    (,,) <$> peek pa <*> peek pt <*> peek pr
