/*
 * crtm_gpu.h - C-ABI of the GB300 library for CRTM's per-profile x channel
 * forward, K-matrix, adjoint and tangent-linear path (ODPS absorption, cloud
 * and aerosol scattering, Emission / ADA / SOI solvers).
 *
 * Each entry point stands in for one reference interface (paths relative to
 * the JCSDA/CRTMv3 source tree):
 *
 *   crtm_gpu_init        CRTM_Init        src/CRTM_LifeCycle.f90:520-576
 *   crtm_gpu_destroy     CRTM_Destroy     src/CRTM_LifeCycle.f90:1131
 *   crtm_gpu_forward     CRTM_Forward     src/CRTM_Forward_Module.f90:229-245
 *   crtm_gpu_k_matrix    CRTM_K_Matrix    src/CRTM_K_Matrix_Module.f90:300-322
 *   crtm_gpu_adjoint     CRTM_Adjoint     src/CRTM_Adjoint_Module.f90:299-309
 *   crtm_gpu_tangent_linear  CRTM_Tangent_Linear  src/CRTM_Tangent_Linear_Module.f90:271
 *   crtm_gpu_last_error  Display_Message  src/Utility/Message_Handler.f90:114
 *
 * Status codes are the reference's (Message_Handler.f90:27-31).  A call fails
 * as a whole when any profile fails (CRTM_Forward_Module.f90:415-421); the
 * per-profile status words say which.
 *
 * Data layout (structure of arrays, C order, profiles outermost).  Layer 0
 * is the top layer.  Every array is indexed with the batch's max_layers
 * stride; layers past a profile's n_layers are ignored on input and written
 * as zero on output.
 *
 *   level_pressure [P][max_layers+1] hPa     pressure, temperature [P][max_layers]
 *   absorber       [P][n_absorbers][max_layers]  (units as the reference's Absorber_Units)
 *   surface / geometry fields [P]; emissivity [P][n_channels] (Options%Emissivity)
 *   radiance, brightness_temperature [P][n_channels]
 *   K-matrix: temperature [P][n_channels][max_layers],
 *             absorber [P][n_channels][n_absorbers][max_layers],
 *             water_temperature, surface_emissivity [P][n_channels]
 *   adjoint:  temperature [P][max_layers], absorber [P][n_absorbers][max_layers],
 *             water_temperature [P]
 *
 * Outputs are overwritten (the reference accumulates into caller-zeroed
 * K/AD structures; a caller that wants accumulation adds the result).
 *
 * Threading: calls on one handle are serialised on the handle's CUDA stream;
 * separate handles may be used from separate host threads.
 */
#ifndef CRTM_GPU_H
#define CRTM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define CRTM_GPU_SUCCESS 0
#define CRTM_GPU_INFORMATION 1
#define CRTM_GPU_WARNING 2
#define CRTM_GPU_FAILURE 3

/* Arithmetic forms.  FP64: every stage in double precision.  MIXED: predictors,
 * regression, gas layer optics, the scattering layers' MOM solver, layer
 * records, adding and their reverse sweeps in single precision; Map_Input,
 * the Planck inversion (radiance to brightness temperature), the surface
 * terms, the cloud/aerosol LUT lookups and their derivatives, the adding's
 * matrix inversions, the OPTRAN term and the SOI solver in double precision,
 * as are the scattering layers that single precision cannot resolve (nearly
 * conservative, or with a nearly defective MOM eigenbasis).  Outputs are
 * double precision in both forms; the mixed form keeps 0.01 K in brightness
 * temperatures and 1e-3 of the largest Jacobian. */
#define CRTM_GPU_FP64 0
#define CRTM_GPU_MIXED 1

typedef struct crtm_gpu_context* crtm_gpu_handle;

typedef struct {
  int n_profiles;
  int max_layers;
  const int* n_layers;            /* [P] */
  int n_absorbers;
  const int* absorber_id;         /* [n_absorbers] HITRAN ids (H2O=1, CO2=2, O3=3, ...) */
  const double* level_pressure;   /* [P][max_layers+1] */
  const double* pressure;         /* [P][max_layers] */
  const double* temperature;      /* [P][max_layers] */
  const double* absorber;         /* [P][n_absorbers][max_layers] */
  /* surface (CRTM_Surface_type) [P] */
  const double* land_coverage;
  const double* water_coverage;
  const double* snow_coverage;
  const double* ice_coverage;
  const double* land_temperature;
  const double* water_temperature;
  const double* snow_temperature;
  const double* ice_temperature;
  /* geometry (CRTM_Geometry_type) [P], degrees */
  const double* sensor_zenith_angle;
  const double* source_zenith_angle;
  const double* surface_altitude; /* may be NULL (0) */
  /* options (CRTM_Options_type): Use_Emissivity is required in this build */
  /* Options%Emissivity [P][n_channels] (Use_Emissivity), or NULL: the
   * emissivity comes from the IR sea-surface model (CRTM_IRSSEM with the
   * handle's Nalli.IRwater.EmisCoeff.bin) at the sensor zenith angle, for
   * infrared sensors, clear-sky batches and water coverage 1 only. */
  const double* emissivity;
  /* clouds (CRTM_Cloud_type, Atmosphere%Cloud(:)).  max_clouds = 0: clear-sky
   * batch, the cloud pointers are not read.  A profile with n_clouds > 0 is
   * solved with the scattering solver (ADA or SOI); its cloud coverage
   * follows cloud_fraction below. */
  int max_clouds;                 /* NC: stride of the cloud arrays */
  const int* n_clouds;            /* [P] clouds of each profile, <= NC */
  const int* cloud_type;          /* [P][NC] WATER=1 ICE=2 RAIN=3 SNOW=4 GRAUPEL=5 HAIL=6 */
  const double* cloud_water_content;    /* [P][NC][max_layers] kg/m^2 */
  const double* cloud_effective_radius; /* [P][NC][max_layers] microns */
  /* Options%n_Streams for profiles with Options%Use_N_Streams (2, 4, 6, 8 or
   * 16), 0 for the reference's stream rule; NULL: the rule everywhere. */
  const int* n_streams;           /* [P] */
  /* Options%RT_Algorithm_Id for cloudy profiles: 56 ADA, 168 SOI
   * (src/CRTM_Parameters.f90:247-248); NULL: ADA everywhere. */
  const int* rt_algorithm_id;     /* [P] */
  /* aerosols (CRTM_Aerosol_type, Atmosphere%Aerosol(:)), in the handle's
   * AerosolCoeff scheme (crtm_gpu_init_aerosol); max_aerosols = 0: none.
   * Aerosols scatter for infrared, visible and ultraviolet sensors only (the
   * reference skips them for microwave). */
  int max_aerosols;               /* NA: stride of the aerosol arrays */
  const int* n_aerosols;          /* [P] aerosols of each profile, <= NA */
  const int* aerosol_type;        /* [P][NA] AerosolCoeff Type ids */
  const double* aerosol_concentration;    /* [P][NA][max_layers] kg/m^2 */
  const double* aerosol_effective_radius; /* [P][NA][max_layers] microns */
  /* Atmosphere%Cloud_Fraction (CRTM_Atmosphere_Define.f90).  Where it is
   * below 1e-12 the layer's clouds are dropped (CRTM_Forward_Module.f90:367-376);
   * a profile with a cloudy layer whose fraction is above 1e-6 is FRACTIONAL
   * (CRTM_Atmosphere.f90:158-203): its radiance is (1 - tcc) x the clear
   * column (gas only, Emission) + tcc x the cloudy column with the water
   * content divided by tcc, tcc the total cloud cover of the overlap scheme
   * (CRTM_CloudCover_Define.f90:447-642).  NULL: 1 in every layer (one cloudy
   * column: tcc = 1 for every overlap scheme). */
  const double* cloud_fraction;   /* [P][max_layers] */
  /* Options%Overlap_Id: 1 maximum, 2 random, 3 maximum-random, 4 average,
   * 5 overcast; NULL: 4 (the reference's default). */
  const int* overlap_id;          /* [P] */
  /* Atmosphere%Aerosol(n)%Effective_Variance (the 'CMAQ' table's sigma axis)
   * and Atmosphere%Relative_Humidity (0-1, the 'GOCART-GEOS5' / 'NAAPS' RH
   * axis), read by those schemes only (CRTM_AerosolScatter.f90:245-252).
   * NULL: zero, as the reference initialises them; the LUT lookup clamps
   * each to its axis. */
  const double* aerosol_effective_variance; /* [P][NA][max_layers] */
  const double* relative_humidity;          /* [P][max_layers] */
  /* Surface%Wind_Speed [P] m/s, read by the IR sea-surface emissivity model
   * (NULL: the reference's default 5 m/s, CRTM_Surface_Define.f90:183). */
  const double* wind_speed;
} crtm_gpu_batch;

typedef struct {
  double* radiance;                /* [P][L] */
  double* brightness_temperature;  /* [P][L] */
  int* status;                     /* [P] per-profile status bits, or NULL */
  /* The other RTSolution components the reference fills on this path
   * (CRTM_RTSolution_Define.f90:201-245), each NULL when not wanted; [P][L]
   * unless noted, layer arrays [P][L][max_layers] on the batch's layers
   * (zero past a profile's n_layers).  Thermal sources only: the solar,
   * visible and active-sensor components stay with the reference.
   *   tb_clear, r_clear: a fractional profile's clear column
   *     (CRTM_Forward_Module.f90:1108-1114); a profile without clouds, or
   *     whose total cloud cover is below 1e-12, its own brightness
   *     temperature and radiance (:1115-1119); zero otherwise.
   *   total_cloud_cover: a fractional profile's (:1092); zero otherwise.
   *   sod: vertically integrated scattering optical depth, the sum of the
   *     layers' scattering coefficients before the delta truncation
   *     (CRTM_AtmOptics.f90:425-427; :978 of the forward module); zero for a
   *     profile without clouds and aerosols.
   *   surface_emissivity: the emissivity used (Common_RTSolution.f90:433).
   *   up_radiance, down_radiance, surface_planck_radiance: the Emission
   *     solver's atmospheric upwelling radiance at the top, downwelling
   *     radiance at the surface and surface Planck radiance
   *     (Common_RTSolution.f90:1195-1198); zero for a profile solved with
   *     ADA or SOI, as in the reference.
   *   n_full_streams: Options%n_Streams + 2, else the stream rule's count
   *     + 2 for a profile with clouds or aerosols, else 0
   *     (CRTM_Forward_Module.f90:866-874, CRTM_RTSolution.f90:1204-1260).
   *   layer_optical_depth: the layers' optical depth after the AtmOptics
   *     combine (Common_RTSolution.f90:239).
   *   upwelling_radiance, upwelling_overcast_radiance: the Emission solver's
   *     upwelling radiance at each layer's bottom and the top-of-atmosphere
   *     radiance of a black cloud filling each layer (Emission_Module.f90:
   *     132,166-172; Common_RTSolution.f90:1206-1207); zero for a profile
   *     solved with ADA or SOI. */
  double* tb_clear;
  double* r_clear;
  double* total_cloud_cover;
  double* sod;
  double* surface_emissivity;
  double* up_radiance;
  double* down_radiance;
  double* surface_planck_radiance;
  int* n_full_streams;
  double* layer_optical_depth;          /* [P][L][max_layers] */
  double* upwelling_radiance;           /* [P][L][max_layers] */
  double* upwelling_overcast_radiance;  /* [P][L][max_layers] */
} crtm_gpu_rtsolution;

typedef struct {
  double* temperature;        /* [P][L][max_layers] */
  double* absorber;           /* [P][L][n_k][max_layers], n_k = n_k_absorbers or n_absorbers */
  double* water_temperature;  /* [P][L] Surface_K%Water_Temperature */
  double* surface_emissivity; /* [P][L] RTSolution_K%Surface_Emissivity */
  /* Optional selection of absorber Jacobians: when n_k_absorbers > 0 only the
   * user absorbers k_absorber_index[0..n_k_absorbers-1] (host pointer, 0-based
   * indices into the batch's absorbers) are written, in that order.  The
   * reference always fills Atmosphere_K%Absorber for every absorber; callers
   * that use only some of them save the rest of the output traffic. */
  int n_k_absorbers;
  const int* k_absorber_index;
  /* Jacobians of scattering profiles (Atmosphere_K%Cloud(n)%Water_Content,
   * %Effective_Radius, Atmosphere_K%Cloud_Fraction, Atmosphere_K%Aerosol(n)%
   * Concentration, %Effective_Radius); each may be NULL (not computed).  Cloud
   * arrays [P][L][max_clouds][max_layers], cloud_fraction [P][L][max_layers],
   * aerosol arrays [P][L][max_aerosols][max_layers]; zero outside each
   * profile's clouds, aerosols and layers. */
  double* cloud_water_content;
  double* cloud_effective_radius;
  double* cloud_fraction;
  double* aerosol_concentration;
  double* aerosol_effective_radius;
  /* Surface_K%Land_Temperature, %Snow_Temperature, %Ice_Temperature [P][L]
   * (each cover's coverage x dBT/dTs, CRTM_Compute_SurfaceT_AD), or NULL */
  double* land_temperature;
  double* snow_temperature;
  double* ice_temperature;
  /* Atmosphere_K%Aerosol(n)%Effective_Variance [P][L][max_aerosols][max_layers]
   * ('CMAQ') and Atmosphere_K%Relative_Humidity [P][L][max_layers]
   * ('GOCART-GEOS5', 'NAAPS'), or NULL; zero under the other schemes. */
  double* aerosol_effective_variance;
  double* relative_humidity;
  /* Surface_K%Wind_Speed [P][L] through the IR sea-surface emissivity model
   * (batch emissivity NULL), or NULL; a 'Nalli2' table's temperature
   * dependence is added into water_temperature. */
  double* wind_speed;
} crtm_gpu_kmatrix;

typedef struct {
  double* temperature;        /* [P][max_layers] */
  double* absorber;           /* [P][n_absorbers][max_layers] */
  double* water_temperature;  /* [P] */
  /* adjoints of the scattering inputs (Atmosphere_AD%Cloud(n)%..., %Cloud_Fraction,
   * %Aerosol(n)%...), each may be NULL: [P][max_clouds][max_layers],
   * [P][max_layers], [P][max_aerosols][max_layers] */
  double* cloud_water_content;
  double* cloud_effective_radius;
  double* cloud_fraction;
  double* aerosol_concentration;
  double* aerosol_effective_radius;
  double* land_temperature;   /* [P] Surface_AD%Land_Temperature, or NULL */
  double* snow_temperature;   /* [P] */
  double* ice_temperature;    /* [P] */
  double* aerosol_effective_variance; /* [P][max_aerosols][max_layers], or NULL */
  double* relative_humidity;          /* [P][max_layers], or NULL */
  double* wind_speed;                 /* [P] Surface_AD%Wind_Speed (emissivity model), or NULL */
} crtm_gpu_adjoint_out;

/* Tangent-linear inputs (Atmosphere_TL, Surface_TL and the emissivity
 * perturbation): each array may be NULL (no perturbation of that input).
 * Shapes as the batch's: temperature [P][max_layers], absorber
 * [P][n_absorbers][max_layers], cover temperatures [P], emissivity [P][L],
 * cloud arrays [P][max_clouds][max_layers], cloud_fraction [P][max_layers],
 * aerosol arrays [P][max_aerosols][max_layers]. */
typedef struct {
  const double* temperature;
  const double* absorber;
  const double* land_temperature;
  const double* water_temperature;
  const double* snow_temperature;
  const double* ice_temperature;
  const double* emissivity;
  const double* cloud_water_content;
  const double* cloud_effective_radius;
  const double* cloud_fraction;
  const double* aerosol_concentration;
  const double* aerosol_effective_radius;
  const double* aerosol_effective_variance; /* [P][max_aerosols][max_layers] */
  const double* relative_humidity;          /* [P][max_layers] */
  const double* wind_speed;                 /* [P] (emissivity model) */
} crtm_gpu_tl_in;

/* CRTM_Init: loads <coeff_path>/<sensor_id>.SpcCoeff.bin and .TauCoeff.bin
 * (ODPS) for each sensor, and <coeff_path>/CloudCoeff.bin, AerosolCoeff.bin
 * and Nalli.IRwater.EmisCoeff.bin when those files exist (the reference's
 * default file names), and uploads them to the current CUDA device.  Batches
 * with clouds or aerosols need the matching LUT; batches without an
 * emissivity need the IR water table. */
int crtm_gpu_init(const char* coeff_path, int n_sensors, const char* const* sensor_ids,
                  crtm_gpu_handle* handle);

/* CRTM_Init with its Aerosol_Model and AerosolCoeff_File arguments
 * (src/CRTM_LifeCycle.f90:523-561,678,706): aerosol_model 'CRTM' (the
 * default), 'CMAQ', 'GOCART-GEOS5' or 'NAAPS' selects the LUT layout and
 * interpolation (CRTM_AerosolScatter.f90:822-918); aerosol_coeff_file is the
 * LUT's file name under coeff_path (NULL: AerosolCoeff.bin).  NULL
 * aerosol_model means 'CRTM'. */
int crtm_gpu_init_aerosol(const char* coeff_path, int n_sensors, const char* const* sensor_ids,
                          const char* aerosol_model, const char* aerosol_coeff_file,
                          crtm_gpu_handle* handle);

/* CRTM_Destroy */
int crtm_gpu_destroy(crtm_gpu_handle handle);

/* Number of channels of sensor index `sensor` (0-based, init order) that
 * calls process (all of the coefficient files' channels unless a subset is
 * set), or -1 (CRTM_ChannelInfo_n_Channels, ChannelInfo/
 * CRTM_ChannelInfo_Define.f90:336-340). */
int crtm_gpu_n_channels(crtm_gpu_handle handle, int sensor);

/* CRTM_ChannelInfo_Subset (ChannelInfo/CRTM_ChannelInfo_Define.f90:444-517):
 * later calls for `sensor` process only the n channels at the 0-based file
 * positions channel_index[0..n-1], in file order; their outputs have n
 * channels ([P][n]...), as do the emissivity and seed inputs.  n = 0: no
 * channels (calls return at once); n < 0: all channels again (Reset).
 * Positions out of range or given twice fail and leave the setting as it
 * was.  The call waits for the handle's work in flight. */
int crtm_gpu_set_channel_subset(crtm_gpu_handle handle, int sensor, int n, const int* channel_index);

/* The processed channels' file positions (up to capacity of them written to
 * channel_index, which may be NULL); returns their count, or -1. */
int crtm_gpu_get_channel_subset(crtm_gpu_handle handle, int sensor, int capacity, int* channel_index);

/* Select the arithmetic form for later calls (CRTM_GPU_FP64 or CRTM_GPU_MIXED). */
int crtm_gpu_set_precision(crtm_gpu_handle handle, int precision);

/* CRTM_Forward for one sensor: host buffers.  Profiles with clouds or
 * aerosols use the ADA or SOI scattering solver (Options%RT_Algorithm_Id),
 * as do the K-matrix, adjoint and tangent-linear entry points. */
int crtm_gpu_forward(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                     crtm_gpu_rtsolution* rts);

/* CRTM_K_Matrix for one sensor: host buffers.  bt_k [P][L] is the
 * RTSolution_K%Brightness_Temperature seed (NULL means 1 everywhere). */
int crtm_gpu_k_matrix(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                      const double* bt_k, crtm_gpu_kmatrix* k, crtm_gpu_rtsolution* rts);

/* CRTM_Adjoint for one sensor: host buffers; bt_ad [P][L] seeds. */
int crtm_gpu_adjoint(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                     const double* bt_ad, crtm_gpu_adjoint_out* ad, crtm_gpu_rtsolution* rts);

/* CRTM_Tangent_Linear: the forward radiances and brightness temperatures
 * (rts) and the brightness-temperature perturbation bt_tl [P][L] produced by
 * the input perturbations tl.  Computed as the K-matrix contracted with the
 * perturbations (exact to rounding; it costs about one K-matrix call and keeps
 * the K-matrix in device scratch owned by the handle). */
int crtm_gpu_tangent_linear(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                            const crtm_gpu_tl_in* tl, crtm_gpu_rtsolution* rts, double* bt_tl);

/* Device-resident variants: every pointer in batch / outputs is a device
 * pointer of the handle's device; `stream` is the cudaStream_t the work is
 * enqueued on (NULL: CUDA's default stream, so the work is ordered with the
 * caller's default-stream work).  They return after enqueueing the work. */
int crtm_gpu_forward_device(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                            crtm_gpu_rtsolution* rts, void* stream);
int crtm_gpu_k_matrix_device(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                             const double* bt_k, crtm_gpu_kmatrix* k, crtm_gpu_rtsolution* rts,
                             void* stream);
int crtm_gpu_adjoint_device(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                            const double* bt_ad, crtm_gpu_adjoint_out* ad,
                            crtm_gpu_rtsolution* rts, void* stream);
int crtm_gpu_tangent_linear_device(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                                   const crtm_gpu_tl_in* tl, crtm_gpu_rtsolution* rts, double* bt_tl,
                                   void* stream);

/* No counterpart in the reference (CRTM_Tangent_Linear and CRTM_Adjoint run
 * the forward model again on every call).  A variational inner loop applies
 * the tangent linear and the adjoint many times about one trajectory:
 * crtm_gpu_linearize evaluates the trajectory's forward (rts) and its
 * K-matrix once, for every input the batch has, into device memory owned by
 * the handle (device buffers, enqueued on `stream`); then
 * crtm_gpu_tangent_linear_apply gives bt_tl [P][L] for perturbations tl, and
 * crtm_gpu_adjoint_apply the outputs of CRTM_Adjoint for a seed bt_ad [P][L],
 * each as one contraction with the stored Jacobians (the same numbers as
 * crtm_gpu_tangent_linear / crtm_gpu_adjoint about that trajectory, to
 * rounding).  All pointers are device pointers; tl and ad have the
 * trajectory batch's shapes.  A later linearize or tangent-linear call
 * replaces the trajectory, and a channel-subset change of its sensor ends it;
 * profiles whose trajectory status was not 0 give 0.
 * The apply calls fail when they ask for a Jacobian the trajectory does not
 * hold (for example cloud perturbations of a batch without clouds). */
int crtm_gpu_linearize(crtm_gpu_handle handle, int sensor, const crtm_gpu_batch* batch,
                       crtm_gpu_rtsolution* rts, void* stream);
int crtm_gpu_tangent_linear_apply(crtm_gpu_handle handle, const crtm_gpu_tl_in* tl, double* bt_tl,
                                  void* stream);
int crtm_gpu_adjoint_apply(crtm_gpu_handle handle, const double* bt_ad, crtm_gpu_adjoint_out* ad,
                           void* stream);

/* No counterpart in the reference (CRTM_K_Matrix allocates its work arrays on
 * every call).  crtm_gpu_k_matrix_device without device-memory allocation:
 * the intermediates live in a static per-device scratch of
 * CRTM_GPU_STATIC_SCRATCH_MIB MiB, for callers whose device memory is held by
 * another allocator or who cannot afford the device-wide synchronisation of
 * cudaMalloc/cudaFree inside a call.  Batches are processed in chunks that fit
 * the scratch; a call fails (CRTM_GPU_FAILURE, message from
 * crtm_gpu_last_error) when one profile's intermediates do not fit.  With no
 * batch emissivity, the IR sea-surface emissivity model's 3 x P x L doubles
 * also come from the scratch (the call fails when they leave no room for one
 * profile).  crtm_gpu_init looks up the scratch address on its device (the
 * module's first use there); where it has not, the first call on a device
 * does.  The entry points are not safe to capture into a CUDA graph: each
 * call reads host tables (absorber maps, bucket counts) while it enqueues its
 * work.  The scratch is shared by all handles on a device: calls that overlap
 * in time race and must be ordered by the caller. */
#define CRTM_GPU_STATIC_SCRATCH_MIB 128
int crtm_gpu_k_matrix_device_static(crtm_gpu_handle handle, int sensor,
                                    const crtm_gpu_batch* batch, const double* bt_k,
                                    crtm_gpu_kmatrix* k, crtm_gpu_rtsolution* rts, void* stream);

/* Tuning of the pipeline (no reference counterpart: the reference's only
 * batching parameter is the OpenMP chunking of profiles and channels,
 * CRTM_Forward_Module.f90:328-357).  Kept per sensor and per arithmetic form
 * (CRTM_GPU_FP64 / CRTM_GPU_MIXED).  Neither setting changes any output's
 * arithmetic, only the work decomposition:
 *   map_channels    channels per map_kernel CTA: 8, 16 or 32; 0 = the handle
 *                   default (16, or the CRTM_GPU_MAP_CHANNELS environment
 *                   variable); reduced automatically when the tiles exceed
 *                   the shared-memory budget
 *   chunk_profiles  at most this many profiles per pipeline pass; 0 = as many
 *                   as the workspace budget holds (the static-scratch entry
 *                   point sizes its own passes and ignores it)
 *   ms_per_call     the autotuner's measured time of one call with this
 *                   setting; 0 when set by crtm_gpu_set_tuning
 * crtm_gpu_get_tuning reports the values in effect (map_channels resolved). */
typedef struct {
  int map_channels;
  int chunk_profiles;
  double ms_per_call;
} crtm_gpu_tuning;
int crtm_gpu_get_tuning(crtm_gpu_handle handle, int sensor, int precision, crtm_gpu_tuning* out);
int crtm_gpu_set_tuning(crtm_gpu_handle handle, int sensor, int precision, const crtm_gpu_tuning* t);

/* Autotuner (no reference counterpart).  Runs crtm_gpu_k_matrix_device on the
 * given device buffers under each candidate tuning (map_channels 16, 8, 32,
 * each with no chunk cap, P/2 and P/4; duplicates dropped), once untimed and
 * then `reps` (1..1000) times between CUDA events on `stream`, and keeps the
 * fastest for the sensor and the form the call runs in.  Up to max_trials
 * measured candidates go to `trials` (may be NULL), their number to *n_trials
 * and the winner to *chosen (either may be NULL).  On return the outputs hold
 * the batch's K-matrix and RTSolution.  On failure the previous tuning is
 * kept. */
int crtm_gpu_autotune_k_matrix_device(crtm_gpu_handle handle, int sensor,
                                      const crtm_gpu_batch* batch, const double* bt_k,
                                      crtm_gpu_kmatrix* k, crtm_gpu_rtsolution* rts, void* stream,
                                      int reps, crtm_gpu_tuning* trials, int max_trials,
                                      int* n_trials, crtm_gpu_tuning* chosen);

/* Copy the last error message of the handle (or of the last failed init when
 * handle is NULL) into buf; returns its length. */
int crtm_gpu_last_error(crtm_gpu_handle handle, char* buf, int n);

/* Number of kernel launches the handle has issued since creation. */
long long crtm_gpu_launch_count(crtm_gpu_handle handle);

/* Stage timing (no reference counterpart; the reference's only timing hook is
 * the compile-time enable_timing flag, CRTM_Forward_Module.f90:265).  When
 * enabled, every kernel launch is bracketed by CUDA events on the launch
 * stream.  crtm_gpu_stage_times synchronises the handle's pending work and
 * returns, per stage, the accumulated milliseconds and launch counts since the
 * last reset: stages 0 prep, 1 absorb_fwd, 2 column, 3 absorb_ad, 4 map_out,
 * 5 adjoint_sum, 6 scatter_layers (layer records), 7 scatter_adding (adding or
 * orders of interaction and their adjoints), 8 scatter_contract (record
 * adjoints contracted with the layer optics' derivatives), 9 scatter_species
 * (cover chain rule and the species outputs).  Returns the number of stages. */
int crtm_gpu_set_profiling(crtm_gpu_handle handle, int enable);
int crtm_gpu_stage_times(crtm_gpu_handle handle, double* ms, long long* launches, int n, int reset);

#ifdef __cplusplus
}
#endif
#endif
