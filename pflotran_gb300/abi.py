"""ctypes mirror of include/pfchem.h (the C ABI of the GPU chemistry library).

The field order and types must match the header exactly; tests/test_abi.py
checks the structure sizes against the C compiler's view of the header.
"""
import ctypes as C

PFCHEM_MAX_PRI = 16
PFCHEM_MAX_CPLX = 64
PFCHEM_MAX_MNRL = 16
PFCHEM_MAX_IONX = 8
PFCHEM_MAX_SRFRXN = 8
PFCHEM_MAX_SRFCPLX = 32
PFCHEM_MAX_NNZ = 8
PFCHEM_MAX_PREF = 4
PFCHEM_MAX_PREF_SPEC = 4

ACT_COEF_FREQUENCY_OFF = 0
ACT_COEF_FREQUENCY_TIMESTEP = 1
ACT_COEF_FREQUENCY_NEWTON_ITER = 2
ACT_COEF_ALGORITHM_LAG = 3
ACT_COEF_ALGORITHM_NEWTON = 4

NULL_SURFACE = 0
COLLOID_SURFACE = 1
MINERAL_SURFACE = 2
ROCK_SURFACE = 3

RESIDUAL_ABSOLUTE = 0
RESIDUAL_RELATIVE = 1
ACCUM_DT_CONSISTENT = 0
ACCUM_LITERAL = 1

CELL_CONVERGED = 0
CELL_MAXITER = 1
CELL_SINGULAR = 2
CELL_NONFINITE = 3
CELL_INNER_MAXITER = 4
CELL_INACTIVE = 5

KERNEL_SPECIALIZED = 0
KERNEL_GENERIC = 1
KERNEL_SPECIALIZED_COMPACT = 2
KERNEL_COOP8 = 3
KERNEL_COOP16 = 4
KERNEL_COOP32 = 5
JACOBIAN_REFERENCE = 0
JACOBIAN_EXACT = 1
MLP_MMA_SYNC = 0
MLP_TCGEN05 = 1

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)


class Network(C.Structure):
    _fields_ = [
        ("naqcomp", C.c_int32), ("neqcplx", C.c_int32), ("nkinmnrl", C.c_int32),
        ("neqionxrxn", C.c_int32), ("nsrfcplxrxn", C.c_int32), ("nsrfcplx", C.c_int32),
        ("eqcplx_ld", C.c_int32), ("kinmnrl_ld", C.c_int32), ("eqionx_ld", C.c_int32),
        ("srfcplxrxn_ld", C.c_int32), ("srfcplx_ld", C.c_int32),
        ("max_num_prefactors", C.c_int32), ("max_num_prefactor_species", C.c_int32),
        ("reserved0", C.c_int32),
        ("primary_spec_Z", _f64p), ("primary_spec_a0", _f64p),
        ("eqcplxspecid", _i32p), ("eqcplxstoich", _f64p), ("eqcplxh2oid", _i32p),
        ("eqcplxh2ostoich", _f64p), ("eqcplx_Z", _f64p), ("eqcplx_a0", _f64p),
        ("eqcplx_logK", _f64p), ("eqcplx_logKcoef", _f64p),
        ("debyeA", C.c_double), ("debyeB", C.c_double), ("debyeBdot", C.c_double),
        ("kinmnrlspecid", _i32p), ("kinmnrlstoich", _f64p), ("kinmnrlh2oid", _i32p),
        ("kinmnrlh2ostoich", _f64p), ("kinmnrl_logK", _f64p), ("kinmnrl_logKcoef", _f64p),
        ("kinmnrl_rate_constant", _f64p), ("kinmnrl_activation_energy", _f64p),
        ("kinmnrl_molar_vol", _f64p), ("kinmnrl_affinity_threshold", _f64p),
        ("kinmnrl_rate_limiter", _f64p), ("kinmnrl_Temkin_const", _f64p),
        ("kinmnrl_min_scale_factor", _f64p), ("kinmnrl_affinity_power", _f64p),
        ("kinmnrl_num_prefactors", _i32p), ("kinmnrl_pref_rate", _f64p),
        ("kinmnrl_pref_activation_energy", _f64p), ("kinmnrl_prefactor_id", _i32p),
        ("kinmnrl_pref_alpha", _f64p), ("kinmnrl_pref_beta", _f64p),
        ("kinmnrl_pref_atten_coef", _f64p),
        ("eqionx_rxn_cationid", _i32p), ("eqionx_rxn_k", _f64p), ("eqionx_rxn_CEC", _f64p),
        ("eqionx_rxn_to_surf", _i32p), ("eqionx_rxn_Z_flag", _i32p),
        ("srfcplxrxn_to_complex", _i32p), ("srfcplxrxn_surf_type", _i32p),
        ("srfcplxrxn_to_surf", _i32p), ("srfcplxrxn_site_density", _f64p),
        ("srfcplxrxn_stoich_flag", _i32p), ("srfcplxspecid", _i32p), ("srfcplxstoich", _f64p),
        ("srfcplxh2oid", _i32p), ("srfcplxh2ostoich", _f64p),
        ("srfcplx_free_site_stoich", _f64p), ("srfcplx_logK", _f64p), ("srfcplx_logKcoef", _f64p),
    ]


class Options(C.Structure):
    _fields_ = [
        ("use_log_formulation", C.c_int32), ("act_coef_update_frequency", C.c_int32),
        ("act_coef_update_algorithm", C.c_int32), ("use_activity_h2o", C.c_int32),
        ("use_isothermal", C.c_int32), ("residual_tol_kind", C.c_int32),
        ("accum_mode", C.c_int32), ("max_iterations", C.c_int32),
        ("max_dlnC", C.c_double), ("max_relative_change_tolerance", C.c_double),
        ("max_residual_tolerance", C.c_double),
        ("update_kinetic_state", C.c_int32), ("jacobian", C.c_int32),
        ("exact_jacobian_after", C.c_int32), ("reserved3", C.c_int32),
    ]


class Cells(C.Structure):
    _fields_ = [
        ("ncells", C.c_int64), ("on_device", C.c_int32), ("reserved2", C.c_int32),
        ("temperature", C.c_void_p), ("saturation", C.c_void_p), ("den_kg", C.c_void_p),
        ("porosity", C.c_void_p), ("volume", C.c_void_p), ("soil_particle_density", C.c_void_p),
        ("active", C.c_void_p), ("total", C.c_void_p),
        ("pri_molal", C.c_void_p), ("ionic_strength", C.c_void_p), ("ln_act_h2o", C.c_void_p),
        ("mnrl_volfrac", C.c_void_p), ("mnrl_area", C.c_void_p), ("total_sorb_eq", C.c_void_p),
        ("eqionx_ref_cation_sorbed_conc", C.c_void_p), ("srfcplxrxn_free_site_conc", C.c_void_p),
        ("total_out", C.c_void_p), ("mnrl_rate", C.c_void_p), ("sec_molal", C.c_void_p),
        ("iterations", C.c_void_p), ("status", C.c_void_p),
        ("alt_guess", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("ncells", C.c_int64), ("sum_iterations", C.c_int64), ("max_iterations", C.c_int32),
        ("nonconverged", C.c_int32), ("alt_guess_used", C.c_int64), ("kernel_ms", C.c_double),
        ("lane_slots", C.c_int64), ("drain_ms", C.c_double),
    ]


class Launch(C.Structure):
    _fields_ = [
        ("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
        ("refill_min_idle", C.c_int32), ("variant", C.c_int32),
    ]


CELL_FIELDS_IN = ("temperature", "saturation", "den_kg", "porosity", "volume",
                  "soil_particle_density", "active", "total")
CELL_FIELDS_STATE = ("pri_molal", "ionic_strength", "ln_act_h2o", "mnrl_volfrac", "mnrl_area",
                     "total_sorb_eq", "eqionx_ref_cation_sorbed_conc", "srfcplxrxn_free_site_conc")
CELL_FIELDS_OUT = ("total_out", "mnrl_rate", "sec_molal", "iterations", "status", "alt_guess")


class ReactionBlocksOut(C.Structure):
    """pfchem_reaction_blocks_out."""
    _fields_ = [("res", C.c_void_p), ("jac", C.c_void_p), ("total", C.c_void_p), ("dtotal", C.c_void_p),
                ("total_sorb", C.c_void_p), ("dtotal_sorb", C.c_void_p)]


class MineralUpdate(C.Structure):
    """pfchem_mineral_update."""
    _fields_ = [("update_porosity", C.c_int32), ("update_surface_area", C.c_int32),
                ("surface_area_with_porosity", C.c_int32), ("reserved", C.c_int32),
                ("minimum_porosity", C.c_double), ("surf_area_vol_frac_pwr", C.c_void_p),
                ("surf_area_porosity_pwr", C.c_void_p), ("mnrl_volfrac0", C.c_void_p), ("mnrl_area0", C.c_void_p),
                ("porosity0", C.c_void_p), ("porosity", C.c_void_p),
                ("armor_crit_vol_frac", C.c_void_p), ("armor_mineral", C.c_void_p), ("armor_flag", C.c_int32),
                ("reserved2", C.c_int32), ("armor_flag_out", C.c_void_p)]


def mineral_update(arrays, update_porosity=1, update_surface_area=1, surface_area_with_porosity=0,
                   minimum_porosity=0.0, armor_flag=0):
    """MineralUpdate over `arrays` (dict of numpy arrays or torch tensors keyed
    by the pointer fields, armor_flag_out a host int32 numpy array); the
    arrays must stay alive while it is used."""
    def ptr(k):
        a = arrays.get(k)
        if a is None:
            return None
        return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data
    return MineralUpdate(update_porosity, update_surface_area, surface_area_with_porosity, 0, minimum_porosity,
                         ptr("surf_area_vol_frac_pwr"), ptr("surf_area_porosity_pwr"), ptr("mnrl_volfrac0"),
                         ptr("mnrl_area0"), ptr("porosity0"), ptr("porosity"), ptr("armor_crit_vol_frac"),
                         ptr("armor_mineral"), int(armor_flag), 0, ptr("armor_flag_out"))

CONSTRAINT_TOTAL, CONSTRAINT_FREE, CONSTRAINT_CHARGE_BAL, CONSTRAINT_PH, CONSTRAINT_LOG, CONSTRAINT_MINERAL = 1, 2, 3, 4, 5, 6
CONSTRAINT_GAS, CONSTRAINT_TOTAL_SORB = 7, 8
PFCHEM_MAX_GAS_ROWS = 8


class Constraint(C.Structure):
    """pfchem_constraint."""
    _fields_ = [("type", C.c_void_p), ("mineral", C.c_void_p), ("value", C.c_void_p),
                ("max_iterations", C.c_int32), ("npassive_gas", C.c_int32), ("paseq_ld", C.c_int32),
                ("reserved", C.c_int32), ("paseqspecid", C.c_void_p), ("paseqstoich", C.c_void_p),
                ("paseqh2oid", C.c_void_p), ("paseqh2ostoich", C.c_void_p), ("paseqlogK", C.c_void_p),
                ("paseqlogKcoef", C.c_void_p)]


def constraint(types, values_ptr, spec_ids=None, max_iterations=0, gases=None):
    """Constraint over numpy `types` / `spec_ids` (int32) and a values
    pointer; `gases` the dict of GasTable.arrays() (kept alive by the caller)."""
    def p(a):
        return None if a is None else a.ctypes.data
    g = gases or {}
    return Constraint(p(types), p(spec_ids), values_ptr, int(max_iterations), int(g.get("n", 0)),
                      int(g.get("ld", 0)), 0, p(g.get("specid")), p(g.get("stoich")), p(g.get("h2oid")),
                      p(g.get("h2ostoich")), p(g.get("logK")), p(g.get("logKcoef")))
