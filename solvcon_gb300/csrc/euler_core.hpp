#pragma once

/*
 * Host object of the GPU Euler core: owns the device mesh, the CE geometry,
 * the solution records and the boundary registry of one mesh, and runs the
 * march on one CUDA stream.  It mirrors solvcon's EulerCore
 * (cpp/solvcon/multidim/euler.hpp:56-211) operation for operation.
 */

#include "common.hpp"
#include "mesh_host.hpp"

#include <cstdint>
#include <memory>
#include <vector>

namespace scg
{

// Array ids of the EulerCore surface (wrap_multidim.cpp:381-408 order).
enum EulerArray : int
{
    EA_CEVOL = 0,
    EA_CECND = 1,
    EA_SFCND = 2,
    EA_SFNML = 3,
    EA_SO0C = 4,
    EA_SO0N = 5,
    EA_SO0T = 6,
    EA_SO1C = 7,
    EA_SO1N = 8,
    EA_STM = 9,
    EA_CFLO = 10,
    EA_CFLC = 11,
    EA_GAMMA = 12,
    EA_COUNT = 13,
};

// Operation ids (EulerCore methods without arguments).
enum EulerOp : int
{
    EO_PREPARE_CE = 0,
    EO_UPDATE = 1,
    EO_CALC_SOLT = 2,
    EO_CALC_SOLN = 3,
    EO_BC_SOLN = 4,
    EO_CALC_CFL = 5,
    EO_CALC_DSOLN = 6,
    EO_BC_DSOLN = 7,
    EO_MARCH_SUBSTEP = 8,
    // Not a reference operation: the solution state back to that of a new
    // core (records, CFL numbers, gamma, limiter mask and stm zero; buffer
    // bookkeeping reset), the mesh, geometry and boundary conditions kept.
    EO_RESET_STATE = 9,
};

enum EulerBCKind : int
{
    BC_NONREFL = 0,
    BC_SLIPWALL = 1,
    BC_INLET = 2,
};

// Scalar fields of the newest solution over the body cells, derived on the
// device (the properties of EulerField, solvcon/multidim/euler/_field.py).
enum EulerField : int
{
    EF_DENSITY = 0,
    EF_VELX = 1,
    EF_VELY = 2,
    EF_VELZ = 3,
    EF_SPEED = 4,
    EF_PRESSURE = 5,
    EF_MACH = 6,
    EF_TOTAL_ENERGY = 7,
    EF_CFL = 8,
    EF_COUNT = 9,
};

// Precision of the march: state/flux arithmetic and stored geometry.
enum Precision : int
{
    PREC_FP64 = 0,         // everything FP64 (the reference's arithmetic)
    PREC_FP32_GEOM64 = 1,  // FP32 state and flux, FP64 geometry in HBM (the FP32 form)
    PREC_FP32 = 2,         // FP32 state and flux, FP64-computed geometry stored FP32 (faster variant)
};

struct EulerBoundary
{
    int kind;
    std::vector<int32_t> faces;
    std::vector<double> value;
};

class EulerCoreBase
{
public:
    virtual ~EulerCoreBase() = default;

    int ndim = 0;
    int64_t ncell = 0, ngstcell = 0;
    int neq = 0;
    double time_increment = 0.0;
    double sigma0 = 3.0, taumin = 0.0, tauscale = 1.0;
    int precision = PREC_FP64;
    int single_ct = -1; // the cell type if every body cell has it, else -1

    // Array shape in the reference layout; nghost is the first-axis ghost count.
    void array_shape(int which, int64_t * shape, int * nd, int64_t * nghost) const;
    int64_t array_size(int which) const;

    virtual void get_array(int which, double * out) = 0;
    virtual void set_array(int which, double const * in) = 0;
    virtual void init_solution(double gamma, double rho, double const * v, double p) = 0;
    virtual void op(int which) = 0;
    virtual void march(int64_t steps) = 0;
    // set_array(EA_SO0N, so0n), set_array(EA_SO1N, so1n), march(steps), with
    // the upload overlapped with the first substep when both tables are
    // whole-array ranges of scg_host_alloc blocks.
    virtual void march_from_host(double const * so0n, double const * so1n, int64_t steps) = 0;
    // Have every later march also leave array `which` (EA_SO0N or EA_SO1N)
    // of its last substep in the host block `host` (a whole-array, 16-byte
    // aligned range of one scg_host_alloc block): written by the last FP64
    // substep kernel itself, or by a gather queued after an FP32 march;
    // host = nullptr stops it.
    virtual void deliver(int which, double * host, int64_t count) = 0;
    // True while a delivery registered with deliver() is still valid.
    virtual bool delivering() = 0;
    virtual void sync() = 0;
    virtual void set_stream(cudaStream_t s) = 0;
    virtual void limiter_mask(uint8_t * out) = 0;
    // FP64 totals of so0n[:, i] * clvol over body cells (Kahan-summed blocks).
    virtual void totals(double * out) = 0;
    // min and max of cflo over body cells.
    virtual void cfl_range(double * out) = 0;
    // One EulerField scalar over the body cells, FP64, into host out[ncell].
    virtual void field(int which, double * out) = 0;

    // Raw device view of the newest order-0 solution (so0n rows inside the
    // solution records), the cell volumes and the core's stream.
    struct StateView
    {
        void const * rec;     // record buffer holding so0n
        int rec_stride;       // reals per record
        int neq;
        bool fp32;            // records hold float instead of double
        double const * clvol; // [ngstcell + ncell]
        int64_t ncell, ngstcell;
        cudaStream_t stream;
        void const * comp;    // FP32: rounding residual of so0n [neq][ncell], or null
    };
    virtual StateView state_view() = 0;

    // Batched march support (batch.cu).  batch_begin() leaves the core ready
    // for fused substeps run by someone else: boundary tables uploaded and the
    // next substep's so0t computed.  fill_args() writes the kernel argument
    // block (dev::MarchArgs<R, G>) of the substep whose current buffer is
    // cur ^ offset into out (size bytes).  batch_end(steps) records that
    // `steps` full steps ran.
    virtual void batch_begin() = 0;
    virtual void fill_args(int offset, void * out, size_t size) = 0;
    virtual void batch_end(int64_t steps) = 0;
    virtual size_t device_bytes() const = 0;
    virtual cudaStream_t get_stream() const = 0;
    // Per-launch CUDA-event timing of the fused substep kernel.
    virtual void profile(bool on) = 0;
    virtual void profile_stats(double * ms_total, int64_t * launches) = 0;

    void add_bc(int kind, std::vector<int32_t> const & faces, std::vector<double> const & value);
    void clear_bc();
    void normal_matrix(int32_t ifc, double * out) const;
    std::vector<EulerBoundary> const & boundaries() const { return m_bcs; }

protected:
    // Host copies of the mesh tables the boundary registry needs.
    int64_t m_nface = 0, m_ngstface = 0;
    std::vector<int32_t> m_fccls; // full, ghost rows first
    std::vector<double> m_fcnml;  // full, ghost rows first
    std::vector<EulerBoundary> m_bcs;
    bool m_bc_dirty = true;
    std::vector<double> m_stm; // the reference's unused scratch table
};

std::unique_ptr<EulerCoreBase> make_euler_core(HostMesh const & mesh, double time_increment, int precision);

} // namespace scg

// The opaque handle behind scg_euler* in include/scg.h.
struct scg_euler
{
    std::unique_ptr<scg::EulerCoreBase> c;
};
