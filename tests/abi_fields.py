"""Field list for the byte-layout check of include/ppf_gb300.h against the
reference's crates/ppf-cts-solver/src/cpp/data.hpp.

Each entry is (reference struct, field path); the header's struct of the same
layout is named 'Ppf' + reference name.
"""
import subprocess
import tempfile
from pathlib import Path

STRUCTS = {
    "VertexParam": ["ghat", "offset", "friction"],
    "EdgeParam": ["stiffness", "bend", "ghat", "offset", "friction", "strainlimit",
                  "plasticity", "plasticity_threshold", "bend_rest_from_geometry",
                  "deform_damping", "bend_damping"],
    "FaceParam": ["model", "mu", "lambda", "friction", "ghat", "offset", "bend",
                  "strainlimit", "shrink_x", "shrink_y", "pressure", "plasticity",
                  "plasticity_threshold", "bend_plasticity", "bend_plasticity_threshold",
                  "bend_rest_from_geometry", "deform_damping", "bend_damping",
                  "bend_warp", "bend_weft"],
    "HingeParam": ["bend", "ghat", "offset", "plasticity", "plasticity_threshold",
                   "bend_damping", "bend_warp", "bend_weft"],
    "TetParam": ["model", "mu", "lambda", "shrink", "plasticity",
                 "plasticity_threshold", "deform_damping"],
    "VertexProp": ["area", "volume", "mass", "rest_bend_angle", "fix_index",
                   "pull_index", "param_index", "pdrd_body_index", "collider"],
    "EdgeProp": ["length", "initial_length", "mass", "fixed", "param_index"],
    "FaceProp": ["area", "mass", "fixed", "rest_excluded", "collider", "param_index"],
    "HingeProp": ["length", "area", "rest_angle", "uv_edge_sin2", "fixed",
                  "collider", "param_index"],
    "TetProp": ["mass", "volume", "fixed", "rest_excluded", "param_index"],
    "PdrdBodyProp": ["rest_centroid", "rest_gram_inv", "volume", "vertex_start",
                     "vertex_count", "mass_per_vertex", "joint_mode", "joint_axis",
                     "joint_pin"],
    "FixPair": ["position", "step_delta", "ghat", "index", "kinematic"],
    "PullPair": ["position", "weight", "index"],
    "TorqueGroup": ["axis_component", "vertex_start", "vertex_count", "hint_vertex"],
    "TorqueVertex": ["magnitude", "index", "group_id"],
    "Stitch": ["index", "weight", "stiffness"],
    "Sphere": ["center", "ghat", "friction", "radius", "thickness", "bowl",
               "reverse", "kinematic"],
    "Floor": ["ground", "ghat", "friction", "thickness", "up", "kinematic"],
    "TranslationLock": ["axis", "total_mass", "pdrd_body_index", "dmap_index",
                        "rotation_axis", "rotation_mode", "anchor"],
    "CollisionMesh": ["vertex", "face", "edge", "prop.vertex", "prop.face",
                      "prop.edge", "param_arrays.vertex", "param_arrays.face",
                      "param_arrays.edge", "neighbor.vertex", "neighbor.hinge",
                      "neighbor.edge"],
    "Constraint": ["fix", "pull", "torque_groups", "torque_vertices", "sphere",
                   "floor", "stitch", "mesh"],
    "RestShapeUpdate": ["inv_rest2x2", "inv_rest3x3", "exclude_face", "exclude_tet"],
    "ParamSet": ["time", "air_friction", "air_density", "constraint_tol", "prev_dt",
                 "dt", "playback", "min_newton_steps", "target_toi",
                 "stitch_length_factor", "cg_max_iter", "cg_tol",
                 "line_search_max_t", "ccd_eps", "max_dx", "eiganalysis_eps",
                 "friction_eps", "isotropic_air_friction", "gravity", "wind",
                 "barrier", "friction_mode", "csrmat_max_nnz", "fix_xz",
                 "disable_contact", "inactive_momentum", "precond",
                 "schwarz_levels", "max_newton_steps", "disable_pin_dof_removal"],
    "StepResult": ["time", "ccd_success", "pcg_success", "intersection_free",
                   "newton_progress", "pin_feasible", "contact_separated"],
    "IntersectionRecord": ["type", "elem0", "elem1", "num_verts0", "num_verts1",
                           "positions"],
    "DataSet": ["vertex", "vertex.prev", "vertex.curr", "mesh", "mesh.mesh.face",
                "mesh.mesh.hinge", "mesh.mesh.edge", "mesh.mesh.tet",
                "mesh.neighbor.vertex.face", "mesh.neighbor.vertex.hinge",
                "mesh.neighbor.vertex.edge", "mesh.neighbor.vertex.rod",
                "mesh.neighbor.hinge.face", "mesh.neighbor.edge.face",
                "mesh.type.face", "mesh.type.vertex", "mesh.type.hinge", "prop",
                "prop.vertex", "prop.edge", "prop.face", "prop.hinge", "prop.tet",
                "prop.pdrd_body", "param_arrays", "param_arrays.vertex",
                "param_arrays.edge", "param_arrays.face", "param_arrays.hinge",
                "param_arrays.tet", "inv_rest2x2", "inv_rest3x3", "constraint",
                "constraint.mesh", "fixed_index_table", "transpose_table",
                "rod_count", "shell_face_count", "surface_vert_count",
                "pdrd_vert_list", "pdrd_rest_centered", "grain_omega",
                "grain_inv_inertia", "grain_torque", "grain_ang_stiff",
                "grain_contact_normal", "grain_inv_inertia_center",
                "grain_omega_prev", "grain_A", "grain_B", "grain_grot",
                "tet_hess_slots", "face_hess_slots", "edge_hess_slots",
                "hinge_hess_slots", "rod_bend_hess_slots", "stitch_hess_slots",
                "translation_lock", "translation_lock_index",
                "translation_lock_initial", "statistics_object_index",
                "statistics_static_object_index", "statistics_contact_count"],
}


def program(header_lines, prefix):
    out = list(header_lines)
    out += ["#include <cstdio>", "#include <cstddef>", "int main() {", 'std::printf("{");',
            "int first = 1;"]
    for s, fields in STRUCTS.items():
        t = prefix + s
        out.append(f'std::printf("%s\\"{s}\\": %zu", first ? "" : ", ", sizeof({t})); first = 0;')
        for f in fields:
            out.append(f'std::printf(", \\"{s}.{f}\\": %zu", offsetof({t}, {f}));')
    out += ['std::printf("}\\n");', "return 0; }"]
    return "\n".join(out) + "\n"


def measure(header_lines, prefix, include_dirs, extra_flags=()):
    import json

    src = program(header_lines, prefix)
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "layout.cpp"
        exe = Path(d) / "layout"
        c.write_text(src)
        cmd = ["g++", "-std=c++17", "-Wno-invalid-offsetof", *extra_flags,
               *[f"-I{p}" for p in include_dirs], str(c), "-o", str(exe)]
        subprocess.run(cmd, check=True, capture_output=True)
        r = subprocess.run([str(exe)], check=True, capture_output=True, text=True)
        return json.loads(r.stdout)
