"""Drop-in import path of the reference (``exafac``), served by rdist_tensor_gb300."""
