"""Small scene files for the scene-file reader's accept/reject cases.

Each entry: name -> file text ("@DIR@" stands for the directory the files are
written to).  Shared by make_golden.py (which records the reference's verdict
on each) and tests/test_scene_file.py.  None of them reads a mesh or an IBL
but "missing_mesh", whose mesh does not exist.
"""
import os
import shutil

import numpy as np

_SPHERE = "Sphere {\n  Radius: 1\n  Position: 0, 0, 0\n  Material: 0, 0, 0, LAMBERT, 0.5, 0.5, 0.5\n}\n"

CASES = {
    "minimal": "Objects:\n" + _SPHERE,
    "no_header_values": "# only a comment\n\nObjects:\n" + _SPHERE,
    "basedir_slash": "BaseDir: @DIR@/\nObjects:\n" + _SPHERE,
    "unknown_header_key": "Camera: 1\nObjects:\n" + _SPHERE,
    "no_objects_line": "Base Dir: @DIR@\n" + _SPHERE,
    "objects_last_line": "Base Dir: @DIR@\nObjects:",
    "nothing_after_objects": "Objects:\n",
    "nested_block": "Objects:\nSphere {\nSphere {\n}\n}\n",
    "unknown_type": "Objects:\nCube {\n}\n",
    "close_without_open": "Objects:\n}\n",
    "short_material": "Objects:\nSphere {\n  Radius: 1\n  Material: 0, 0, 0, LAMBERT, 0.5, 0.5\n}\n",
    "bad_reflection_type": "Objects:\nSphere {\n  Radius: 1\n  Material: 0, 0, 0, METAL, 0.5, 0.5, 0.5\n}\n",
    "refraction_without_ior": "Objects:\nSphere {\n  Radius: 1\n  Material: 0, 0, 0, REFRACTION, 1, 1, 1\n}\n",
    "rates_mismatch": ("Objects:\nSphere {\n  Radius: 1\n  Material: 0, 0, 0, LAMBERT, 0.5, 0.5, 0.5\n"
                       "  Material: 0, 0, 0, SPECULAR, 1, 1, 1\n  MaterialRates: 1, 2, 3\n}\n"),
    "position_two_numbers": ("Objects:\nSphere {\n  Radius: 1\n  Position: 1, 2\n"
                             "  Material: 0, 0, 0, LAMBERT, 0.5, 0.5, 0.5\n}\n"),
    "floor_size_three": ("Objects:\nFloor {\n  Size: 1, 2, 3\n"
                         "  Material: 0, 0, 0, LAMBERT, 0.5, 0.5, 0.5\n}\n"),
    "missing_mesh": "Base Dir: @DIR@\nObjects:\nObj Mesh {\n  FileName: no_such_mesh.obj\n}\n",
    "unclosed_block_at_end": "Objects:\n" + _SPHERE + "Sphere {\n  Radius: 2\n",
    "text_outside_blocks": "Objects:\nstray text: 1\n" + _SPHERE,
    "crlf_free_trailing_blanks": "Objects:\n" + _SPHERE + "\n\n   \n",
    "type_suffix_blanks": "Objects:\nSphereLight   {\n  Radius: 1\n  Material: 1, 1, 1, LAMBERT, 0, 0, 0\n}\n",
    "comment_inside_block": ("Objects:\nSphere {\n  # a comment\n  Radius: 3\n"
                             "  Material: 0, 0, 0, SPECULAR, 1, 1, 1\n}\n"),
}


GOLDEN = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def write(name, directory):
    path = os.path.join(directory, name + ".scene")
    with open(path, "w") as fh:
        fh.write(CASES[name].replace("@DIR@", directory))
    return path


def stage_scene_dir(directory):
    """The files the full scene reads, laid out under directory: full.scene
    (Base Dir = directory), obj/mesh.obj + .mtl, and sky.hdr (the run-length
    encoded .hdr of image_codec.npz)."""
    os.makedirs(os.path.join(directory, "obj"), exist_ok=True)
    for f in ("mesh.obj", "mesh.mtl"):
        shutil.copy(os.path.join(GOLDEN, "obj", f), os.path.join(directory, "obj", f))
    codec = np.load(os.path.join(GOLDEN, "image_codec.npz"))
    with open(os.path.join(directory, "sky.hdr"), "wb") as fh:
        fh.write(codec["hdr_rle_file"].tobytes())
    text = open(os.path.join(GOLDEN, "scene", "full.scene.in")).read().replace("@DIR@", directory)
    path = os.path.join(directory, "full.scene")
    with open(path, "w") as fh:
        fh.write(text)
    return path
