/*
 * rewl.h -- C ABI of the GB300 replica-exchange Wang-Landau (REWL) engine.
 *
 * One engine runs a batch of REWL instances on one GPU.  An instance is one
 * model (2D Ising or 2D Ashkin-Teller with optional random Baxter fields) on an
 * L x L periodic lattice, its energy range cut into overlapping windows
 * (glazier, equal windows) with `replicas_per_window` walkers each.  Every
 * walker of every instance advances inside the same kernel launches; replica
 * exchange, window flatness, in-window averaging and the ln f schedule are
 * device kernels.
 *
 * The reference (meese-wj/REWL_Simulator) has no FFI; its hot path is driven by
 * REWL_simulation::simulate and the duck-typed Hamiltonian plugin surface.  Each
 * entry point below names the reference interface it stands in for.
 *
 * Conventions: plain pointers and sizes; host buffers are owned by the caller
 * and copied synchronously; the engine owns all device memory.  Every function
 * returns REWL_OK or an error code; rewl_last_error_string() describes the last
 * error of the calling thread.  An engine is driven by one host thread at a time.
 */
#ifndef REWL_GB300_H
#define REWL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference has none: it prints and, once, calls exit(1),
 * src/util/vector_matching.hpp:61-65) */
#define REWL_OK 0
#define REWL_EINVAL 22      /* bad descriptor or argument (incl. windows that do not overlap) */
#define REWL_ENOMEM 12      /* device or host allocation failed */
#define REWL_ETIMEDOUT 110  /* rewl_run_cycles deadline passed (host-side, no device wait) */
#define REWL_EDEVICE 1001   /* CUDA runtime error */
#define REWL_EBOUNDS 1002   /* a device-side bounds check fired (energy left its window) */
#define REWL_ESTATE 1003    /* call not valid in the engine's current state */

/* models (compile-time switch in the reference: src/Hamiltonians/model_hamiltonians.hpp:6-40) */
#define REWL_MODEL_ISING2D 0
#define REWL_MODEL_ASHKIN_TELLER2D 1

/* flatness rules (src/REWL/rewl_histograms.hpp:115-152) */
#define REWL_FLAT_MIN_OVER_MEAN 0   /* min H >= p * mean H over valid bins (the usual "flatness 0.8") */
#define REWL_FLAT_MAX_MIN_RATIO 1   /* (max - min)/min <= p in float (reference classic rule) */
#define REWL_FLAT_ALL_VISITED 2     /* every valid bin visited (reference ONE_OVER_T rule) */

/* which bins count for flatness */
#define REWL_MASK_STATIC 0          /* all bins except those holding only impossible energies */
#define REWL_MASK_VISITED 1         /* additionally only bins some replica of the window ever visited */

/* random streams */
#define REWL_RNG_PHILOX 0           /* one Philox4x32-10 draw per attempted flip (production) */
#define REWL_RNG_REPLAY 1           /* consume a caller-supplied uniform stream with the reference's
                                       draw-on-demand rule (src/REWL/wang_landau.hpp:73) */

typedef struct rewl_instance_desc {
    int32_t model;                /* REWL_MODEL_* */
    int32_t L;                    /* linear size, 2..128 (System_Parameters::L) */
    double J;                     /* nearest-neighbour coupling (Ising: integer) */
    double K;                     /* four-spin coupling (Ashkin-Teller only), multiple of 2^-20 */
    const double* fields;         /* Ashkin-Teller Baxter field h_i per site, or NULL; rounded to 2^-20 */
    double energy_min;            /* global energy range [energy_min, energy_max) */
    double energy_max;
    double bin_width;             /* Ising: power of two; Ashkin-Teller: 1/n or power of two */
    int32_t num_windows;          /* glazier windows (src/REWL/glazier.hpp:70-115) */
    int32_t replicas_per_window;  /* REWL_Parameters::replicas_per_window, 1..64 */
    double window_overlap;        /* REWL_Parameters::window_overlap */
    int32_t init_mode;            /* 0: spins uniform +-1 from the seed; 1: all +1 */
    int32_t reserved;
    uint64_t seed;                /* seed of this instance's walkers: the Philox key is its SplitMix64 mix,
                                     so nearby seeds give unrelated walker streams */
} rewl_instance_desc;

typedef struct rewl_batch_desc {
    int32_t num_instances;
    int32_t sweeps_per_exchange;  /* REWL_Parameters::sweeps_per_exchange */
    int32_t sweeps_per_check;     /* REWL_Parameters::sweeps_per_check (multiple of sweeps_per_exchange) */
    int32_t flatness_mode;        /* REWL_FLAT_* */
    double flatness_param;        /* p of the flatness rule */
    double lnf_initial;           /* REWL_Walker::incrementer initial value, (0, 64] */
    double lnf_final;             /* REWL_Parameters::final_increment */
    int32_t mask_mode;            /* REWL_MASK_* */
    int32_t one_over_t;           /* ONE_OVER_T_ALGORITHM switch for the ln f schedule */
    int32_t reduce_logdos;        /* REDUCE_LOGDOS: subtract logdos[0] at each histogram reset */
    int32_t rng_mode;             /* REWL_RNG_* */
    int32_t device;               /* CUDA device ordinal */
    int32_t warps_per_block;      /* 0: automatic; else 1, 2, 4 or 8 */
    int32_t walkers_per_warp;     /* 0: automatic; else 1, 2 or 4 (Ising bin-tracking kernel) */
    int32_t observables;          /* 1: keep per-bin observables (update_observables after every
                                     attempted flip and exchange, rewl_walker.hpp / wang_landau.hpp:51-120);
                                     2: also the G(q_min) Fourier correlators of the reference's default
                                     CORRELATION_LENGTHS build (src/Hamiltonians/Correlations/
                                     fourier_correlator.hpp), one transform at every 1000th count of a bin */
    int32_t graphs;               /* 1: rewl_run_cycles replays each check interval (sweeps, exchanges,
                                     flatness step) as one captured CUDA graph */
    int32_t autotune;             /* 1: the first rewl_run_cycles call runs rewl_autotune first */
    int32_t persistent;           /* 1: every launch group's walkers in one persistent, work-stealing launch
                                     per sweep phase (one walker per warp; Philox streams only) */
    const rewl_instance_desc* instances;
} rewl_batch_desc;

typedef struct rewl_status {
    int64_t sweeps;               /* sweeps done by every walker */
    int64_t cycles;               /* check intervals completed */
    int64_t flat_events;          /* windows that became flat (summed) */
    int64_t windows_done;         /* windows with ln f < lnf_final */
    int64_t windows_total;
    int64_t exchanges_attempted;
    int64_t exchanges_accepted;
    int64_t attempted_flips;      /* single-spin(-flavour) attempts by all walkers */
    int64_t kernel_launches;      /* engine kernels launched since creation */
    int32_t all_done;
    int32_t device_error;         /* device error word (0 = none) */
} rewl_status;

typedef struct rewl_engine rewl_engine;

/* Build the batch on the device: windows, initial lattices, walk into windows.
 * Replaces REWL_simulation's constructor + glazier + adjust_state_to_range
 * (src/Simulation/rewl_simulation.hpp:69-108, src/REWL/rewl_walker.hpp:79-115,
 *  src/Simulation/main.cpp:201-209). */
int rewl_create(const rewl_batch_desc* desc, rewl_engine** out);

/* Free every device allocation (REWL_simulation::~REWL_simulation). */
int rewl_destroy(rewl_engine* eng);

/* Text of the last error raised on the calling thread. */
const char* rewl_last_error_string(void);

/* Sizes and layout.  Walkers are numbered instance-major, then window, then replica
 * (the reference's world rank order, src/REWL/mpi_rewl_comm_setup.hpp:26-77). */
int rewl_num_walkers(const rewl_engine* eng, int32_t* num_walkers);
int rewl_walker_info(const rewl_engine* eng, int32_t walker, int32_t* instance, int32_t* window, int32_t* replica);
int rewl_window_info(const rewl_engine* eng, int32_t instance, int32_t window,
                     double* energy_min, double* energy_max, int32_t* num_bins);

/* Replace a walker's lattice: Ising N spins, Ashkin-Teller sigma plane then tau
 * plane; each entry +1 or -1.  `flavour` is which_to_update (0 sigma, 1 tau).
 * Replaces Hamiltonian::import_DoFs (src/Hamiltonians/Ising2d/ising2d_hamiltonian.hpp:127-133,
 * src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_hamiltonian.hpp:137-143).
 * The energy must lie in the walker's window. */
int rewl_import_dofs(rewl_engine* eng, int32_t walker, const int8_t* dofs, int32_t flavour);

/* Replace an instance's Baxter fields (N doubles, rounded to 2^-20) and recompute
 * every walker's energy.  Replaces Hamiltonian::import_disorder
 * (src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_hamiltonian.hpp:159-165). */
int rewl_import_disorder(rewl_engine* eng, int32_t instance, const double* fields);

/* Random fields as the reference draws them (Disorder::generate_random_field,
 * src/Hamiltonians/Disorder/random_fields.hpp:41-75, with its Gaussian from
 * random_number_generator::get_gaussian, src/util/random_number_generators.hpp:33-57),
 * seeded by the caller instead of the clock: num_sites doubles into out, Gaussian with
 * standard deviation `strength` or uniform on [-2 strength, 2 strength].  Host only (no
 * device needed); feed the result to rewl_instance_desc.fields or rewl_import_disorder. */
#define REWL_DISORDER_UNIFORM 0     /* disorder_distribution::uniform */
#define REWL_DISORDER_GAUSSIAN 1    /* disorder_distribution::gaussian */
int rewl_generate_fields(uint64_t seed, double strength, int32_t distribution, int64_t num_sites, double* out);

/* Set the logDoS of every replica of a window (warm start); values are rounded
 * to the engine's 2^-36 grid and must satisfy |g| <= 2^24 nats (2^60 units).  No reference counterpart (the reference starts at 0,
 * src/REWL/rewl_histograms.hpp:42-50). */
int rewl_set_logdos(rewl_engine* eng, int32_t instance, int32_t window, const double* logdos);

/* Set ln f of a window (REWL_Walker::incrementer, src/REWL/rewl_walker.hpp:21), (0, 64].
 * Sweep launches are sized so that one launch cannot carry a logDoS entry past int64: a
 * large ln f on a large lattice splits an exchange interval into several launches (same
 * results).  A logDoS entry reaching 2^62 units (6.7e7 nats) without a flat event stops the
 * engine with REWL_ESTATE, as does a per-stage count passing 2^32 - 1. */
int rewl_set_lnf(rewl_engine* eng, int32_t instance, int32_t window, double lnf);

/* REWL_RNG_REPLAY only: the uniform stream a walker consumes, one value per
 * uphill in-range attempt (random_number_generator::operator(),
 * src/util/random_number_generators.hpp:29 as used at src/REWL/wang_landau.hpp:73). */
int rewl_set_uniform_stream(rewl_engine* eng, int32_t walker, const double* uniforms, size_t count);

/* Advance every walker by `num_sweeps` sweeps with no exchange and no flatness
 * check (REWL_Walker::wang_landau_walk, src/REWL/rewl_walker.hpp:142-158). */
int rewl_run_sweeps(rewl_engine* eng, int64_t num_sweeps);

/* One replica-exchange round in the current even/odd direction, then flip the
 * direction (REWL_simulation::replica_exchange_update, src/Simulation/rewl_simulation.hpp:228-346). */
int rewl_exchange(rewl_engine* eng);

/* Window flatness vote, in-window logDoS averaging, histogram reset
 * (REDUCE_LOGDOS) and ln f update for every flat window
 * (src/Simulation/rewl_simulation.hpp:361-470,541-600).  `num_flat` may be NULL. */
int rewl_check_flat(rewl_engine* eng, int32_t* num_flat);

/* Zero a window's histograms, optionally subtracting logdos[0] (rewl_histograms::reset_counts,
 * src/REWL/rewl_histograms.hpp:83-95). */
int rewl_reset_histograms(rewl_engine* eng, int32_t instance, int32_t window, int32_t reduce_logdos);

/* Run up to `num_cycles` check intervals, each (sweeps_per_exchange sweeps +
 * exchange) x (sweeps_per_check / sweeps_per_exchange) then the flatness step,
 * stopping early once every window is done or `timeout_ms` (> 0) has passed.
 * The main loop of REWL_simulation::simulate (src/Simulation/rewl_simulation.hpp:473-691). */
int rewl_run_cycles(rewl_engine* eng, int64_t num_cycles, int64_t timeout_ms, rewl_status* status);
/* Time each launch group's admissible kernel shapes (walkers per warp, warps per block) on a
 * few sweeps each (sweeps = 0: about 2e7 attempted flips per trial) and keep the fastest; the
 * engine's state is saved before and restored after, so the simulation is unchanged.  Launch
 * groups (model x kernel x lattice size) of a heterogeneous batch run concurrently on their
 * own streams in every sweep phase. */
int rewl_autotune(rewl_engine* eng, int32_t sweeps);
/* The launch groups' shapes: count rows of [model, bin-tracking kernel, walkers per warp,
 * warps per block]; with shapes NULL or *count too small only *count is set. */
int rewl_launch_shapes(rewl_engine* eng, int32_t* shapes, int32_t* count);

/* Counters; synchronises the engine's stream. */
int rewl_get_status(rewl_engine* eng, rewl_status* status);

/* One walker's lattice (as rewl_import_dofs), state ([E, M] Ising; [E, sigma_mag,
 * tau_mag, baxter, which_to_update] Ashkin-Teller), and its tables: per-stage counts,
 * logDoS, cumulative visits.  Any output pointer may be NULL.
 * (Hamiltonian::current_state / get_front_DoFs, rewl_histograms::export_logdos,
 *  src/REWL/rewl_histograms.hpp:98-104) */
int rewl_export_walker(rewl_engine* eng, int32_t walker, int8_t* dofs, double* state,
                       uint64_t* counts, double* logdos, uint64_t* visits);
/* Per-bin observable averages of one walker (observables = 1 or 2), nb rows of K + 1 doubles: K
 * averages and the number of updates, the layout of the reference's obs_array
 * (Ising2d_Obs, src/Hamiltonians/Ising2d/ising2d_observables.hpp:134-145: K = 3, |m| m^2 m^4;
 * Ashkin_Teller2d_Obs, src/Hamiltonians/Ashkin_Teller2d/ashkin_teller2d_observables.hpp:211-222:
 * K = 12, |s| s^2 s^4 |t| t^2 t^4 |p| p^2 p^4 |b| b^2 b^4 with p^2 = s^2 + t^2).  With
 * observables = 2 the CORRELATION_LENGTHS layout (ising2d_observables.hpp:22-28,
 * ashkin_teller2d_observables.hpp:36-47): Ising K = 4 with G(q_min) after m^4; Ashkin-Teller
 * K = 16 with a G(q_min) after each group of three (sigma, tau computed from sigma as the
 * reference does, phi = their sum, Baxter); G is the mean over the bin's transforms. */
int rewl_export_observables(rewl_engine* eng, int32_t walker, double* out);
/* The same over a window's replicas, weighted by their counts (the final averaging of
 * observables, src/Simulation/rewl_simulation.hpp:361-454). */
int rewl_export_window_observables(rewl_engine* eng, int32_t instance, int32_t window, double* out);

/* A window's logDoS averaged over its replicas with cumulative-visit weights
 * (the final average_and_redistribute_window, src/Simulation/rewl_simulation.hpp:687). */
int rewl_export_window_logdos(rewl_engine* eng, int32_t instance, int32_t window, double* logdos);

/* A window's valid-bin mask (1 byte per bin). */
int rewl_export_window_mask(rewl_engine* eng, int32_t instance, int32_t window, uint8_t* mask);

/* ln f and done flag of a window. */
int rewl_window_state(rewl_engine* eng, int32_t instance, int32_t window, double* lnf, int32_t* done);

/* Concatenate window logDoS tables into one ln g over the instance's energy
 * range and normalise it so that sum_E g(E) = states_per_site^N (minus ln 2 when
 * `half_spectrum`).  Restates concatenate_tables (multiple overlap) and
 * normalize_logDoS (src/util/concatenate_rewl_tables.hpp:167-305,
 * src/util/vector_matching.hpp:38-88, src/util/array_shift.hpp:15-43), splicing
 * where the derivatives differ least (REWL_MATCH_DERIVATIVE below).
 * Masked bins are left out.  On input *count is the capacity of energies/logdos;
 * on output the number of values written. */
int rewl_global_logdos(rewl_engine* eng, int32_t instance, int32_t half_spectrum,
                       double* energies, double* logdos, int32_t* count);

/* The same post-processing on caller-held tables, host only (no engine or device):
 * num_windows windows of sizes[w] rows (ascending energies, valid levels only) stored
 * one after another; consecutive windows must overlap.  The result is normalised to
 * sum g = states_per_site^system_size (halved when half_spectrum).  With num_obs > 0,
 * obs holds num_obs values per row (same order as the energies) and out_obs receives them
 * averaged over each overlap as the reference does (average_two_windows weighted by the
 * number of windows averaged so far, src/util/concatenate_rewl_tables.hpp:42-49,241-256).
 * match selects where neighbouring windows are spliced:
 *   REWL_MATCH_DERIVATIVE: at the overlap bin whose d ln g / dE differ least (the
 *     engine's rule, rewl_global_logdos);
 *   REWL_MATCH_REFERENCE: as the reference's compiled code does, whose abs() of the
 *     derivative difference (src/util/vector_matching.hpp:74,81,83) resolves to the C
 *     library's int abs(int) and so truncates it to an integer: bit for bit the
 *     reference's concatenate_tables + normalize_logDoS.
 * *count: capacity in, rows out. */
#define REWL_MATCH_DERIVATIVE 0
#define REWL_MATCH_REFERENCE 1
int rewl_concatenate_windows(int32_t num_windows, const int32_t* sizes, const double* energies, const double* logdos,
                             int32_t num_obs, const double* obs, double states_per_site, int64_t system_size,
                             int32_t half_spectrum, int32_t match, double* out_energies, double* out_logdos,
                             double* out_obs, int32_t* count);

/* Device time spent in the sweep kernels since the last call (ms) and the
 * number of sweep-kernel launches; timed with CUDA events on the engine stream. */
int rewl_sweep_kernel_time(rewl_engine* eng, double* milliseconds, int64_t* launches);

/* Checkpoint / resume of every mutable device array (lattices, energies, slot
 * mapping, tables, ln f and schedule state, counters).  The reference has no
 * checkpointing (it only prints histograms, src/REWL/rewl_histograms.hpp:155-170).
 * rewl_snapshot_size gives the byte count; rewl_snapshot copies the state into
 * `buffer` (device -> host), rewl_restore copies it back into an engine created
 * from the same descriptor.  Copies are issued on the engine stream; pinned host
 * buffers make them asynchronous DMA transfers.  Both calls synchronise. */
int rewl_snapshot_size(const rewl_engine* eng, size_t* bytes);
int rewl_snapshot(rewl_engine* eng, void* buffer, size_t bytes);
int rewl_restore(rewl_engine* eng, const void* buffer, size_t bytes);

/* The CUDA stream the engine launches on (cudaStream_t as void*). */
int rewl_get_stream(rewl_engine* eng, void** stream);

/* ------------------------------------------------------------------------
 * Learned warm start (no reference counterpart: the reference always starts
 * ln g at 0, src/REWL/rewl_histograms.hpp:42-50).  An MLP maps
 * [E/N, 1/L, J, K, sigma_h, window lo/N, window hi/N] to ln g(E)/N; training
 * and inference run on the GPU with BF16 tensor-core GEMMs (FP32 accumulate).
 * ------------------------------------------------------------------------ */
typedef struct rewl_mlp rewl_mlp;

/* `layers` hidden layers of width `hidden` (multiple of 64), GELU; seeded init. */
int rewl_mlp_create(int32_t device, int32_t hidden, int32_t layers, uint64_t seed, rewl_mlp** out);
int rewl_mlp_destroy(rewl_mlp* mlp);
const char* rewl_mlp_last_error_string(void);
/* number of floats in the (padded) parameter vector */
int rewl_mlp_num_params(const rewl_mlp* mlp, int64_t* count);
/* per layer: input width, output width, weight offset, bias offset (padded layout) */
int rewl_mlp_layout(const rewl_mlp* mlp, int64_t* rows_of_4, int32_t capacity_rows);
/* fp32 master parameters (which = 0) or the last gradient (which = 1) */
int rewl_mlp_get_params(rewl_mlp* mlp, int32_t which, float* out, int64_t count);
int rewl_mlp_set_params(rewl_mlp* mlp, const float* in, int64_t count);
/* y[i] = f(X[i, :in_dim]) for n rows */
int rewl_mlp_predict(rewl_mlp* mlp, const float* X, int32_t n, int32_t in_dim, float* y);
/* one forward + backward of the mean squared error on n rows (n a multiple of 64); no update */
int rewl_mlp_gradient(rewl_mlp* mlp, const float* X, const float* y, int32_t n, int32_t in_dim, float* loss);
/* load a training set into device memory */
int rewl_mlp_set_data(rewl_mlp* mlp, const float* X, const float* y, int32_t n, int32_t in_dim);
/* `steps` Adam steps on random batches of `batch` rows; per-step losses into `losses` (may be NULL) */
int rewl_mlp_train(rewl_mlp* mlp, int32_t steps, int32_t batch, float lr, float* losses);
/* kernels launched by this network so far (updated atomically: calls on one network may come
 * from several threads) */
int rewl_mlp_launches(const rewl_mlp* mlp, int64_t* count);
/* Allocation-free prediction (no counterpart in the reference).  Same result as
 * rewl_mlp_predict, but X (n x in_dim floats) and y (n floats) are DEVICE
 * pointers and the work is enqueued on `stream` (a cudaStream_t; NULL = legacy
 * default stream) without waiting for it.  Activations live in a static 9.5 MiB
 * device array that every GPU loading this library holds until exit, so no call
 * allocates device memory.  It is for callers that cannot call cudaMalloc: a host
 * program whose own allocator already holds the device's memory, a loop at its
 * device-memory limit, or a driver loop that must not stall (cudaMalloc may
 * synchronise the device).  At most 4096 rows per call and hidden width at most
 * 256, else REWL_EINVAL.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress): make it before any stream capture.  The array is shared
 * by all networks on a device and keeps the last call's contents: calls that may
 * overlap on the GPU (other streams, other threads) race and must be ordered by the
 * caller.  Parameters must not change while a call is in flight.  The call does not
 * wait for the GPU, so a tensor-core GEMM whose bounded wait ran out is reported by
 * the next synchronising rewl_mlp_* call (REWL_EDEVICE); until then this call writes
 * NaN to y.  The caller's current device is left as it was. */
int rewl_mlp_predict_noalloc(rewl_mlp* mlp, const float* X, int32_t n, int32_t in_dim, float* y, void* stream);

/* ------------------------------------------------------------------------
 * Canonical thermodynamics from a density of states (FP64 log-sum-exp on the GPU).
 * ------------------------------------------------------------------------ */
const char* rewl_thermo_last_error_string(void);
/* Thermodynamics::calculate_thermodynamics (src/Thermodynamics/thermodynamics.hpp:158-297)
 * for num_T temperatures T_i = Tmin + i (Tmax - Tmin) / num_T: out holds num_T rows of
 * [F, U, U2, S, C, num_obs observables] (per site; column counts_col of obs, if >= 0, is
 * averaged over the bins instead of weighted), temperatures the T_i.  E, lng: nbins values;
 * obs: nbins x num_obs (rewl_export_window_observables layout) or NULL; trapezoid: the
 * reference's TRAPEZOIDAL_RULE (end bins weighted 1/2). */
int rewl_thermodynamics(const double* E, const double* lng, const double* obs, int32_t nbins, int32_t num_obs,
                        int32_t counts_col, double system_size, double Tmin, double Tmax, int32_t num_T,
                        int32_t trapezoid, int32_t device, double* temperatures, double* out);
/* Susceptibility N (<m^2> - <m>^2) / T and Binder cumulants from those rows
 * (order_parameter_cumulants.hpp:17-48).  Ising: 2 values per T (susceptibility, cumulant);
 * Ashkin-Teller: 8 (sigma, tau, Baxter, then phi with the two-component cumulant).  With
 * correlators (rows in the observables = 2 layout) each pair is followed by the correlation
 * length over L, (L / 2 pi) sqrt((<m^2> - <G>) / <G>) / L (order_parameter_cumulants.hpp:52-59;
 * calculate_nonlinear_observables, ising2d_observables.hpp:166-193,
 * ashkin_teller2d_observables.hpp:240-300): Ising 3 values per T, Ashkin-Teller 12. */
int rewl_nonlinear_observables(int32_t model, int32_t correlators, const double* rows, int32_t num_T,
                               int32_t row_len, const double* temperatures, double system_size, double* out);

/* ------------------------------------------------------------------------
 * Output files in the reference's text formats (main.cpp:241-365): '#' header lines
 * naming the columns, comma-delimited rows, std::scientific with 15 digits.
 * names: the column names after the leading ones, separated by '\n'.
 * ------------------------------------------------------------------------ */
/* Observables on the energies of rewl_global_logdos (rows of K + 1: K averages, count),
 * windows combined by the reference's running mean (concatenate_rewl_tables.hpp:241-256). */
int rewl_global_observables(rewl_engine* eng, int32_t instance, double* obs, int32_t* count);
/* microcanonical_observables-<file_string>.txt: E/N, ln g/N, num_obs observables per bin
 * (write_microcanonical_observables.hpp:16-65) */
int rewl_write_microcanonical(const char* dir, const char* file_string, const char* header, const char* names,
                              int32_t num_bins, int32_t num_obs, double system_size, const double* energies,
                              const double* logdos, const double* obs);
/* self_averaged_observables-<file_string>.txt: T and num_cols values per row
 * (write_self_averaged_observables.hpp:15-59) */
int rewl_write_self_averaged(const char* dir, const char* file_string, const char* header, const char* names,
                             int32_t num_T, int32_t num_cols, const double* temperatures, const double* rows);
/* nonlinear_observables-<file_string>.txt (write_nonlinear_observables.hpp:13-57) */
int rewl_write_nonlinear(const char* dir, const char* file_string, const char* header, const char* names,
                         int32_t num_T, int32_t num_cols, const double* temperatures, const double* rows);
/* All three files for one instance: concatenated normalised ln g (+ observables when the engine
 * keeps them), thermodynamics over T_i = Tmin + i (Tmax - Tmin) / num_T on the GPU, and the
 * nonlinear observables (src/Simulation/main.cpp:241-365). */
int rewl_write_outputs(rewl_engine* eng, int32_t instance, const char* dir, const char* file_string,
                       const char* header, double Tmin, double Tmax, int32_t num_T);

#ifdef __cplusplus
}
#endif

#endif /* REWL_GB300_H */
