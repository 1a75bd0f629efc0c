"""Load the self-contained golden fixtures of tests/golden/ back into specs."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCALARS = ["dim", "ldmWgt", "knlOrder", "knlWidth", "knlEps", "spdTanVal", "spdTsvVal", "btmWgt",
           "timeStp", "timeNum", "cgItrMax", "cgTolSqu"]


def names():
    """The whole-model frame cases (frame2d_*, frame3d_*); other fixtures have their own layout."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "frame*.npz")))


def load(name: str):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    obj = {k[4:]: z[k] for k in z.files if k.startswith("obj_")}
    spec = {k: z[k].item() for k in SCALARS}
    spec["dim"] = int(spec["dim"])
    spec["knlOrder"] = int(spec["knlOrder"])
    spec["timeNum"] = int(spec["timeNum"])
    spec["cgItrMax"] = int(spec["cgItrMax"])
    spec.update(elaType="frame", elmObj=obj, lmkIniMat=z["lmkIniMat"], tauPrmVec=z["tauPrmVec"],
                modVec=z["modVec"], ynkActPrmVec=z["ynkActPrmVec"], reaActPrmVec=z["reaActPrmVec"],
                tgt=(z["tgtCen"], z["tgtDir"], z["tgtVol"]))
    v = z["vfdKnl"]
    spec["vfd"] = (chr(int(v[0])), float(v[1]), chr(int(v[2])), float(v[3]))
    ref = dict(tauVarMat=z["tauVarMat"], lmkStk=z["ref_lmkStk"], tauMat=z["ref_tauMat"],
               deformation_obj=z["ref_deformation_obj"], objfcn=z["ref_objfcn"])
    return spec, ref
