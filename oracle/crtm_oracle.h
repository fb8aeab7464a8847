/*
 * CPU FP64 oracle for the CRTM ODPS + Emission forward / K-matrix / adjoint path.
 *
 * TEST INFRASTRUCTURE ONLY: this library is the checker for the GPU library,
 * and the timed CPU baseline of bench.py.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  It is never part of the
 * product path.
 *
 * It restates, from the reference's Fortran behaviour, the routines named in
 * crtm_oracle.c (each function cites the file:line it follows).
 *
 * Parity unpinned: the reference (Fortran 2003, netCDF-Fortran required) has
 * no compiler in this environment and ships no numeric golden vectors for
 * this path (its coefficient files and result files are Git-LFS stubs), so
 * this oracle is pinned by known-answer cases, finite differences and
 * tangent-linear/adjoint symmetry instead of by reference outputs.
 *
 * The batch layout is the one of include/crtm_gpu.h.
 */
#ifndef CRTM_ORACLE_H
#define CRTM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_handle_s or_handle;

/* Load <dir>/<sensor_id>.TauCoeff.bin and .SpcCoeff.bin; returns NULL on error. */
or_handle* or_init(const char* coeff_dir, const char* sensor_id);
void or_destroy(or_handle* h);
int or_n_channels(const or_handle* h);
int or_n_ref_layers(const or_handle* h);
int or_group(const or_handle* h);
const char* or_last_error(void);

typedef struct {
  int n_profiles;
  int max_layers;            /* stride of layer arrays                       */
  const int* n_layers;       /* [P]                                          */
  int n_absorbers;           /* user absorbers                               */
  const int* absorber_id;    /* [Jabs]                                       */
  const double* level_pressure; /* [P][max_layers+1]                         */
  const double* pressure;       /* [P][max_layers]                           */
  const double* temperature;    /* [P][max_layers]                           */
  const double* absorber;       /* [P][Jabs][max_layers]                     */
  const double* surface_land_coverage, *surface_water_coverage,
              * surface_snow_coverage, *surface_ice_coverage;     /* [P] */
  const double* surface_land_temperature, *surface_water_temperature,
              * surface_snow_temperature, *surface_ice_temperature; /* [P] */
  const double* sensor_zenith_angle;   /* [P] degrees */
  const double* source_zenith_angle;   /* [P] degrees */
  const double* surface_altitude;      /* [P] */
  const double* emissivity;            /* [P][L] */
  const int* k_absorber_mask;          /* [Jabs] nonzero: return this absorber's K-matrix / adjoint
                                          (NULL: all); the others stay zero */
} or_batch;

/* Forward: radiance and brightness temperature [P][L]; layer_od [P][L][max_layers] optional. */
int or_forward(const or_handle* h, const or_batch* b, double* radiance, double* bt,
               double* layer_od, int n_threads);

/* K-matrix with seed d(BT)=bt_k[P][L] (NULL: 1).  Outputs, overwritten:
 * temperature_k [P][L][Kmax], absorber_k [P][L][Jabs][Kmax], water_temperature_k [P][L],
 * surface_emissivity_k [P][L]; radiance/bt as in the forward. */
int or_k_matrix(const or_handle* h, const or_batch* b, const double* bt_k,
                double* radiance, double* bt, double* temperature_k, double* absorber_k,
                double* water_temperature_k, double* surface_emissivity_k, int n_threads);

/* Adjoint: like the K-matrix but summed over channels: temperature_ad [P][Kmax],
 * absorber_ad [P][Jabs][Kmax], water_temperature_ad [P]. */
int or_adjoint(const or_handle* h, const or_batch* b, const double* bt_ad,
               double* radiance, double* bt, double* temperature_ad, double* absorber_ad,
               double* water_temperature_ad, int n_threads);

/* Test hook: mapped temperature T[K], absorbers A[Jm][K], secants sec[K] and
 * predictors X[K][J][18] of profile m. */
int or_profile_state(const or_handle* h, const or_batch* b, int m, double* T, double* A,
                     double* sec, double* X);

/* Tangent-linear BT for perturbations of T and absorbers (used by symmetry tests):
 * temperature_tl [P][Kmax], absorber_tl [P][Jabs][Kmax], water_temperature_tl [P];
 * bt_tl [P][L] out.  Computed by central differences of the forward model with step h. */
int or_tangent_fd(const or_handle* hd, const or_batch* b, const double* temperature_tl,
                  const double* absorber_tl, const double* water_temperature_tl, double step,
                  double* bt_tl, int n_threads);

/* ---- clouds and the ADA solver ------------------------------------------- */
typedef struct or_cloud_s or_cloud;

/* Load a CloudCoeff binary file (Release 3). */
or_cloud* or_cloud_init(const char* path);
void or_cloud_destroy(or_cloud* c);

typedef struct {
  int max_clouds;                  /* NC: stride of the cloud arrays            */
  const int* n_clouds;             /* [P] clouds used by each profile (<= NC)   */
  const int* cloud_type;           /* [P][NC] WATER=1 ICE=2 RAIN=3 SNOW=4 GRAUPEL=5 HAIL=6 */
  const double* water_content;     /* [P][NC][max_layers] kg/m^2                */
  const double* effective_radius;  /* [P][NC][max_layers] microns               */
  const int* n_streams;            /* [P] Options%n_Streams, 0 = stream rule; may be NULL */
  const int* rt_algorithm;         /* [P] Options%RT_Algorithm_Id: 56 ADA, 168 SOI; may be NULL (ADA) */
  int max_aerosols;                /* NA: stride of the aerosol arrays (0: none) */
  const int* n_aerosols;           /* [P] */
  const int* aerosol_type;         /* [P][NA] AerosolCoeff Type ids */
  const double* aerosol_concentration;     /* [P][NA][max_layers] kg/m^2 */
  const double* aerosol_effective_radius;  /* [P][NA][max_layers] microns */
  const double* cloud_fraction;    /* [P][max_layers] Cloud_Fraction; NULL: 1 in every layer */
  const int* overlap;              /* [P] Options%Overlap_Id 1-5; NULL: 4 (average) */
  const double* aerosol_effective_variance;  /* [P][NA][max_layers] ('CMAQ'); NULL: 0 */
  const double* relative_humidity; /* [P][max_layers] Atmosphere%Relative_Humidity ('GOCART-GEOS5',
                                      'NAAPS'); NULL: 0 */
} or_clouds;

typedef struct or_aerosol_s or_aerosol;
enum { OR_AEROSOL_CRTM = 0, OR_AEROSOL_CMAQ = 1, OR_AEROSOL_GOCART = 2, OR_AEROSOL_NAAPS = 3 };
/* Load an AerosolCoeff binary file (Release 4) for the scheme 'CRTM',
 * 'CMAQ', 'GOCART-GEOS5' or 'NAAPS' (CRTM_Init's Aerosol_Model). */
or_aerosol* or_aerosol_init_scheme(const char* path, const char* scheme);
/* scheme 'CRTM' */
or_aerosol* or_aerosol_init(const char* path);
void or_aerosol_destroy(or_aerosol* a);

/* Forward with clouds and aerosols: ADA or SOI for profiles with clouds or
 * aerosols, Emission otherwise.  cc / ca may be NULL when unused. */
int or_forward_scatter(const or_handle* h, const or_cloud* cc, const or_aerosol* ca, const or_batch* b,
                       const or_clouds* cl, double* radiance, double* bt, int n_threads);

/* The RTSolution components beyond radiance and brightness temperature,
 * each NULL when not wanted ([P][L]; the layer arrays [P][L][max_layers]),
 * with the meanings of include/crtm_gpu.h's crtm_gpu_rtsolution. */
typedef struct {
  double* tb_clear, *r_clear, *total_cloud_cover, *sod, *surface_emissivity;
  double* up_radiance, *down_radiance, *surface_planck_radiance;
  int* n_full_streams;
  double* layer_optical_depth, *upwelling_radiance, *upwelling_overcast_radiance;
} or_rts_ext;

/* or_forward_scatter with the further RTSolution components of CRTM_Forward
 * (CRTM_Forward_Module.f90:866-874,978,1086-1119; Common_RTSolution.f90:239,
 * 433,1195-1207; Emission_Module.f90:117-172).  cl->max_clouds and
 * max_aerosols may be 0 (a clear-sky batch). */
int or_forward_ext(const or_handle* h, const or_cloud* cc, const or_aerosol* ca, const or_batch* b,
                   const or_clouds* cl, double* radiance, double* bt, const or_rts_ext* x, int n_threads);

/* K-matrix of a batch with clouds and aerosols through ADA (reverse mode of
 * CRTM_ADA_AD / MOM_AD and the scattering, combine and LUT adjoints), with the
 * clear-sky gas chain; outputs as or_k_matrix plus the cloud water content
 * and effective radius Jacobians [P][L][NC][Kmax] and the aerosol
 * concentration and first-coordinate Jacobians [P][L][NA][Kmax] (NULL: not
 * returned).  Profiles on SOI, or fractional ones whose total cloud cover is
 * not 1, are refused. */
int or_k_matrix_scatter(const or_handle* h, const or_cloud* cc, const or_aerosol* ca, const or_batch* b,
                        const or_clouds* cl, const double* bt_k, double* radiance, double* bt,
                        double* temperature_k, double* absorber_k, double* water_temperature_k,
                        double* surface_emissivity_k, double* wc_k, double* re_k, double* ac_k, double* ar_k,
                        int n_threads);

/* ---- IR sea-surface emissivity (CRTM_IRSSEM) ------------------------------ */
typedef struct or_irwater_s or_irwater;
/* Load an IRwaterCoeff binary file (Release 4). */
or_irwater* or_irwater_init(const char* path);
void or_irwater_destroy(or_irwater* w);
/* CRTM_Compute_IRSSEM (CRTM_IRSSEM.f90:204-334) at one angle (degrees):
 * Lagrange interpolation in angle, frequency (cm^-1) and wind speed (m/s),
 * and water temperature (K) for a 'Nalli2' table; each clamped to its axis. */
double or_irssem(const or_irwater* w, double water_temperature, double wind_speed, double frequency,
                 double angle);

/* Test hooks: one ADA layer (row-major nZ x nZ blocks) and the angle/phase setup. */
int or_amom_layer(int nS, int nZ, double w, double tau, const double* mu, const double* wt,
                  const double* ff, const double* bb, double B, double* trans, double* refl,
                  double* src);
int or_phase_setup(int nleg, double mu_sensor, const double* pc, double* mu, double* wt, double* ff,
                   double* bb, int* nZ_out);

/* ---- CRTM_Atmosphere_AddLayers ------------------------------------------- */
/* The layers added above one profile whose top lies below the model's first
 * level (0.005 hPa); returns their number n (0: none can be added). */
int or_add_layers(int nlev, const double* mlp, const double* mlt, const double* mla, int J,
                  double top, const double* up, const double* ut, const double* ua,
                  double* pl, double* p, double* t, double* a);

#ifdef __cplusplus
}
#endif
#endif
