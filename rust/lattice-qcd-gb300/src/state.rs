//! Device-resident lattice states behind the reference's state traits.
use std::cell::OnceCell;
use std::ffi::CStr;
use std::fmt;
use std::os::raw::c_int;
use std::ptr::NonNull;

use lattice_qcd_gb300_sys as sys;
use lattice_qcd_rs::error::{LatticeInitializationError, StateInitializationError};
use lattice_qcd_rs::field::{EField, LinkMatrix, Su3Adjoint};
use lattice_qcd_rs::lattice::{Direction, DirectionList, LatticeCyclic, LatticeLinkCanonical, LatticePoint};
use lattice_qcd_rs::simulation::{
    LatticeState, LatticeStateDefault, LatticeStateEFSyncDefault, LatticeStateNew, LatticeStateWithEField,
    LatticeStateWithEFieldNew, SimulationStateSynchronous,
};
use lattice_qcd_rs::{CMatrix3, Real};
use nalgebra::SVector;

/// Arithmetic of a device state (`lq_precision`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Precision {
    /// FP64 throughout: the reference's results to 1e-12
    F64,
    /// FP32 arithmetic on compensated FP32 storage, FP64 sums
    Mixed,
    /// FP32 arithmetic and storage, FP64 sums
    F32,
}

impl Precision {
    fn raw(self) -> c_int {
        match self {
            Self::F64 => sys::LQ_PRECISION_F64,
            Self::Mixed => sys::LQ_PRECISION_MIXED,
            Self::F32 => sys::LQ_PRECISION_F32,
        }
    }
}

/// A status code of the library other than `LQ_OK`, with the library's last error text.
#[derive(Clone, Debug, PartialEq, Eq)]
pub struct LqError {
    pub code: c_int,
    pub detail: String,
}

impl fmt::Display for LqError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        let name = unsafe { CStr::from_ptr(sys::lq_status_string(self.code)) };
        write!(f, "{} ({})", name.to_string_lossy(), self.detail)
    }
}

impl std::error::Error for LqError {}

pub(crate) fn check(rc: c_int) -> Result<(), LqError> {
    if rc == sys::LQ_OK {
        return Ok(());
    }
    let detail = unsafe { CStr::from_ptr(sys::lq_last_error_string()) }.to_string_lossy().into_owned();
    Err(LqError { code: rc, detail })
}

/// The library's errors in the reference's taxonomy of state construction.
impl From<LqError> for StateInitializationError {
    fn from(e: LqError) -> Self {
        match e.code {
            sys::LQ_ERR_NON_POSITIVE_SIZE => LatticeInitializationError::NonPositiveSize.into(),
            sys::LQ_ERR_DIM_TOO_SMALL => LatticeInitializationError::DimTooSmall.into(),
            sys::LQ_ERR_ZERO_DIMENSION => LatticeInitializationError::ZeroDimension.into(),
            sys::LQ_ERR_GAUSS_PROJECTION => Self::GaussProjectionError,
            _ => Self::IncompatibleSize,
        }
    }
}

/// Owning handle of an `lq_state`.
pub(crate) struct Handle(NonNull<sys::lq_state>);

impl Handle {
    pub(crate) fn create<const D: usize>(lattice: &LatticeCyclic<D>, beta: Real, p: Precision) -> Result<Self, LqError> {
        let mut raw = std::ptr::null_mut();
        check(unsafe {
            sys::lq_state_create(D as c_int, lattice.dim() as c_int, lattice.size(), beta, p.raw(), &mut raw)
        })?;
        Ok(Self(NonNull::new(raw).expect("lq_state_create returned no state")))
    }
    pub(crate) fn ptr(&self) -> *mut sys::lq_state {
        self.0.as_ptr()
    }
    fn try_clone(&self) -> Result<Self, LqError> {
        let mut raw = std::ptr::null_mut();
        check(unsafe { sys::lq_state_clone(self.ptr(), &mut raw) })?;
        Ok(Self(NonNull::new(raw).expect("lq_state_clone returned no state")))
    }
    pub(crate) fn scalar(&self, f: unsafe extern "C" fn(*mut sys::lq_state, *mut f64) -> c_int) -> f64 {
        let mut v = 0.0;
        check(unsafe { f(self.ptr(), &mut v) }).expect("device reduction failed");
        v
    }
    pub(crate) fn t(&self) -> usize {
        let mut t: std::os::raw::c_longlong = 0;
        let null = std::ptr::null_mut();
        check(unsafe { sys::lq_state_info(self.ptr(), null, null, std::ptr::null_mut(), std::ptr::null_mut(), null, std::ptr::null_mut(), &mut t, null) })
            .expect("lq_state_info failed");
        t as usize
    }
}

impl Drop for Handle {
    fn drop(&mut self) {
        unsafe { sys::lq_state_destroy(self.ptr()) };
    }
}

// A handle is used by one thread at a time (the library's rule); moving it between threads is fine.
unsafe impl Send for Handle {}

fn download_links<const D: usize>(h: &Handle, lattice: &LatticeCyclic<D>) -> LinkMatrix {
    let n = lattice.number_of_points() * D;
    let mut data = vec![CMatrix3::zeros(); n];
    // Matrix3<Complex<f64>> is 18 contiguous f64 in column-major order: the serde layout of the ABI
    check(unsafe { sys::lq_links_download(h.ptr(), data.as_mut_ptr().cast(), n * 18) }).expect("lq_links_download");
    LinkMatrix::new(data)
}

fn upload_links(h: &Handle, links: &LinkMatrix) -> Result<(), LqError> {
    check(unsafe { sys::lq_links_upload(h.ptr(), links.as_slice().as_ptr().cast(), links.len() * 18) })
}

/// Links on the device: the place of `LatticeStateDefault<D>`.
pub struct LatticeStateGpu<const D: usize> {
    pub(crate) handle: Handle,
    lattice: LatticeCyclic<D>,
    beta: Real,
    links_mirror: OnceCell<LinkMatrix>,
}

impl<const D: usize> LatticeStateGpu<D> {
    /// `LatticeStateDefault::new_cold` on the device, in the given precision
    pub fn new_cold(lattice: LatticeCyclic<D>, beta: Real, precision: Precision) -> Result<Self, LqError> {
        let handle = Handle::create(&lattice, beta, precision)?;
        Ok(Self { handle, lattice, beta, links_mirror: OnceCell::new() })
    }
    /// `LinkMatrix::new_determinist` drawn on the device from a Philox stream keyed by `seed`
    pub fn new_random(lattice: LatticeCyclic<D>, beta: Real, precision: Precision, seed: u64) -> Result<Self, LqError> {
        let s = Self::new_cold(lattice, beta, precision)?;
        check(unsafe { sys::lq_links_random(s.handle.ptr(), seed) })?;
        Ok(s)
    }
    /// the raw handle, for the entry points beyond the traits
    pub fn as_raw(&self) -> *mut sys::lq_state {
        self.handle.ptr()
    }
    /// the device links changed: the next `link_matrix()` downloads them again
    pub fn invalidate(&mut self) {
        self.links_mirror = OnceCell::new();
    }
    /// `LatticeStateDefault::normalize_link_matrices` (src/simulation/state.rs:754-756)
    pub fn normalize_link_matrices(&mut self) {
        check(unsafe { sys::lq_normalize_link_matrices(self.handle.ptr()) }).expect("lq_normalize_link_matrices");
        self.invalidate();
    }
}

impl<const D: usize> Clone for LatticeStateGpu<D> {
    /// `lq_state_clone`: a device copy of the links (and momenta)
    fn clone(&self) -> Self {
        Self {
            handle: self.handle.try_clone().expect("lq_state_clone"),
            lattice: self.lattice.clone(),
            beta: self.beta,
            links_mirror: OnceCell::new(),
        }
    }
}

impl<const D: usize> LatticeState<D> for LatticeStateGpu<D> {
    const CA: Real = 3_f64;

    fn link_matrix(&self) -> &LinkMatrix {
        self.links_mirror.get_or_init(|| download_links(&self.handle, &self.lattice))
    }

    fn set_link_matrix(&mut self, link_matrix: LinkMatrix) {
        // the reference panics on a size mismatch (src/simulation/state.rs:810-815)
        upload_links(&self.handle, &link_matrix).expect("Link matrices are not of the correct size");
        self.links_mirror = OnceCell::from(link_matrix);
    }

    fn lattice(&self) -> &LatticeCyclic<D> {
        &self.lattice
    }

    fn beta(&self) -> Real {
        self.beta
    }

    fn hamiltonian_links(&self) -> Real {
        self.handle.scalar(sys::lq_hamiltonian_links)
    }
}

impl<const D: usize> LatticeStateNew<D> for LatticeStateGpu<D> {
    type Error = StateInitializationError;

    /// `LatticeStateDefault::new` (src/simulation/state.rs:776-793), FP64 on the device
    fn new(lattice: LatticeCyclic<D>, beta: Real, link_matrix: LinkMatrix) -> Result<Self, Self::Error> {
        if lattice.number_of_canonical_links_space() != link_matrix.len() {
            return Err(StateInitializationError::IncompatibleSize);
        }
        let mut s = Self::new_cold(lattice, beta, Precision::F64)?;
        s.set_link_matrix(link_matrix);
        Ok(s)
    }
}

/// Links and E-field on the device: the place of `LatticeStateEFSyncDefault<LatticeStateDefault<D>, D>`.
pub struct LatticeStateGpuEField<const D: usize> {
    pub(crate) state: LatticeStateGpu<D>,
    e_mirror: OnceCell<EField<D>>,
    /// t of the reference's constructor; the device counts the integration steps after it
    t0: usize,
}

impl<const D: usize> LatticeStateGpuEField<D> {
    /// the state with the momenta dropped (`LatticeStateEFSyncDefault::state_owned`)
    pub fn state_owned(self) -> LatticeStateGpu<D> {
        self.state
    }
    /// a state whose momenta are on the device already (cold after creation)
    pub fn from_state(state: LatticeStateGpu<D>) -> Self {
        Self { state, e_mirror: OnceCell::new(), t0: 0 }
    }
    /// the device fields changed (links and momenta)
    pub fn invalidate(&mut self) {
        self.state.invalidate();
        self.e_mirror = OnceCell::new();
    }
    pub fn as_raw(&self) -> *mut sys::lq_state {
        self.state.as_raw()
    }
}

impl<const D: usize> Clone for LatticeStateGpuEField<D> {
    fn clone(&self) -> Self {
        Self { state: self.state.clone(), e_mirror: OnceCell::new(), t0: self.t0 }
    }
}

impl<const D: usize> LatticeState<D> for LatticeStateGpuEField<D> {
    const CA: Real = 3_f64;

    fn link_matrix(&self) -> &LinkMatrix {
        self.state.link_matrix()
    }
    fn set_link_matrix(&mut self, link_matrix: LinkMatrix) {
        self.state.set_link_matrix(link_matrix);
    }
    fn lattice(&self) -> &LatticeCyclic<D> {
        self.state.lattice()
    }
    fn beta(&self) -> Real {
        self.state.beta()
    }
    fn hamiltonian_links(&self) -> Real {
        self.state.hamiltonian_links()
    }
}

impl<const D: usize> LatticeStateWithEField<D> for LatticeStateGpuEField<D>
where
    Direction<D>: DirectionList,
{
    fn e_field(&self) -> &EField<D> {
        self.e_mirror.get_or_init(|| {
            let n = self.lattice().number_of_points();
            let mut flat = vec![0.0_f64; n * D * 8];
            check(unsafe { sys::lq_efield_download(self.as_raw(), flat.as_mut_ptr(), flat.len()) })
                .expect("lq_efield_download");
            let data = flat
                .chunks(8 * D)
                .map(|site| {
                    SVector::<Su3Adjoint, D>::from_fn(|mu, _| {
                        let mut a = [0.0; 8];
                        a.copy_from_slice(&site[8 * mu..8 * mu + 8]);
                        Su3Adjoint::new_from_array(a)
                    })
                })
                .collect();
            EField::new(data)
        })
    }

    fn set_e_field(&mut self, e_field: EField<D>) {
        let flat: Vec<f64> = e_field
            .data()
            .iter()
            .flat_map(|site| site.iter().flat_map(|a| a.data().iter().copied()).collect::<Vec<f64>>())
            .collect();
        // the reference panics on a size mismatch (src/simulation/state.rs:1394-1399)
        check(unsafe { sys::lq_efield_upload(self.as_raw(), flat.as_ptr(), flat.len()) })
            .expect("E field is not of the correct size");
        self.e_mirror = OnceCell::from(e_field);
    }

    fn t(&self) -> usize {
        self.t0 + self.state.handle.t()
    }

    /// the reference's host function, unchanged (the device computes the same inside its integrator)
    fn derivative_u(
        link: &LatticeLinkCanonical<D>,
        link_matrix: &LinkMatrix,
        e_field: &EField<D>,
        lattice: &LatticeCyclic<D>,
    ) -> Option<CMatrix3> {
        <LatticeStateEFSyncDefault<LatticeStateDefault<D>, D> as LatticeStateWithEField<D>>::derivative_u(
            link, link_matrix, e_field, lattice,
        )
    }

    /// the reference's host function, unchanged
    fn derivative_e(
        point: &LatticePoint<D>,
        link_matrix: &LinkMatrix,
        e_field: &EField<D>,
        lattice: &LatticeCyclic<D>,
    ) -> Option<SVector<Su3Adjoint, D>> {
        <LatticeStateEFSyncDefault<LatticeStateDefault<D>, D> as LatticeStateWithEField<D>>::derivative_e(
            point, link_matrix, e_field, lattice,
        )
    }

    fn hamiltonian_efield(&self) -> Real {
        self.state.handle.scalar(sys::lq_hamiltonian_efield)
    }
}

impl<const D: usize> LatticeStateWithEFieldNew<D> for LatticeStateGpuEField<D>
where
    Direction<D>: DirectionList,
{
    type Error = StateInitializationError;

    /// `LatticeStateEFSyncDefault::new` (src/simulation/state.rs:1330-1361), FP64 on the device
    fn new(
        lattice: LatticeCyclic<D>,
        beta: Real,
        e_field: EField<D>,
        link_matrix: LinkMatrix,
        t: usize,
    ) -> Result<Self, Self::Error> {
        if lattice.number_of_canonical_links_space() != link_matrix.len()
            || lattice.number_of_points() != e_field.len()
        {
            return Err(StateInitializationError::IncompatibleSize);
        }
        let state = LatticeStateGpu::<D>::new(lattice, beta, link_matrix)?;
        let mut s = Self::from_state(state);
        s.set_e_field(e_field);
        s.t0 = t;
        Ok(s)
    }
}

impl<const D: usize> SimulationStateSynchronous<D> for LatticeStateGpuEField<D> where Direction<D>: DirectionList {}
