"""Command-line driver with the reference's flags and output schema
(decompose.py of vbharadwaj-bk/rdist_tensor), running the GB300 engine.

    python decompose.py -i synthetic:planted -t 25 -iter 20 -alg sts_cp \
        -s 65536 -dist accumulator_stationary -e 5

Inputs: the reference's named tensors (HDF5 files, need h5py), ``random``
(the reference's block tensor), or ``synthetic:<planted|zipf4|zipf4_small|zipf5>``.
Extra flags: --seed, --precision {fp64,tf32,bf16}, --factor-file PATH (write the
factors at the end), --init-factors PATH (resume from them).  One process, one GPU.
"""
import argparse
import json
import os
from datetime import datetime

TENSORS = {
    "uber": {"path": "tensors/uber.tns_converted.hdf5", "preprocessing": "none"},
    "patents": {"path": "tensors/patents.tns_converted.hdf5", "preprocessing": "none"},
    "nell1": {"path": "tensors/nell-1.tns_converted.hdf5", "preprocessing": "log_count"},
    "nell2": {"path": "tensors/nell-2.tns_converted.hdf5", "preprocessing": "log_count"},
    "amazon": {"path": "tensors/amazon-reviews.tns_converted.hdf5", "preprocessing": "none"},
    "reddit": {"path": "tensors/reddit-2015.tns_converted.hdf5", "preprocessing": "log_count"},
    "caida": {"path": "tensors/caida_medium.hdf5", "preprocessing": "log_count"},
    "wikidata": {"path": "tensors/wikidata-fixed.tns_converted.hdf5", "preprocessing": "ones"},
}


def decompose(args, output_filename, trial_num):
    from exafac.cpp_ext.py_module import (AccumulatorStationary, CP_ARLS_LEV, ExactALS, LowRankTensor, STS_CP,
                                          TensorStationary)
    from exafac.sparse_tensor_e import DistSparseTensorE, RandomSparseTensor, SyntheticSparseTensor

    if args.input.startswith("random"):
        sparse_tensor = RandomSparseTensor(None, I=10000, N=3, Q=100, seed=args.seed)
    elif args.input.startswith("synthetic:"):
        sparse_tensor = SyntheticSparseTensor(args.input.split(":", 1)[1], seed=args.seed)
    else:
        t = TENSORS[args.input]
        sparse_tensor = DistSparseTensorE(t["path"], None, preprocessing=t["preprocessing"])

    low_rank_tensor = LowRankTensor(args.trank, sparse_tensor.tensor_grid)
    low_rank_tensor.initialize_factors_gaussian_random(seed=args.seed)
    if args.init_factors is not None:  # resume from FACTOR_MODE_i written by --factor-file
        low_rank_tensor.read_from_file(args.init_factors)

    sample_count = 0
    kw = dict(precision=args.precision, seed=args.seed)
    if args.algorithm == "exact":
        optimizer = ExactALS(sparse_tensor.sparse_tensor, low_rank_tensor, **kw)
    elif args.algorithm in ("cp_arls_lev", "sts_cp"):
        if args.samples is None:
            raise ValueError("Must specify a sample count for randomized ALS!")
        if args.distribution is None:
            raise ValueError("Must specify a data distribution for randomized ALS!")
        sample_count = args.samples
        sampler = CP_ARLS_LEV(low_rank_tensor) if args.algorithm == "cp_arls_lev" else STS_CP(low_rank_tensor)
        if args.preprocessing is not None:
            if args.preprocessing != "exact":
                raise ValueError("Unknown preprocessing specification!")
            print("Executing single round of Exact ALS as preprocessing...")
            pre = ExactALS(sparse_tensor.sparse_tensor, low_rank_tensor, precision="fp64", seed=args.seed)
            pre.initialize_ground_truth_for_als()
            pre.execute_ALS_rounds(1, 0, args.epoch_iter)
            pre.deinitialize()
            print("Finished preprocessing...")
        if args.distribution == "accumulator_stationary":
            optimizer = AccumulatorStationary(sparse_tensor.sparse_tensor, low_rank_tensor, sampler,
                                              max_samples=max(sample_count, 1), **kw)
        elif args.distribution == "tensor_stationary":
            optimizer = TensorStationary(sparse_tensor.sparse_tensor, low_rank_tensor, sampler,
                                         max_samples=max(sample_count, 1), **kw)
        else:
            raise ValueError(f"Unrecognized distribution {args.distribution}")
    else:
        raise ValueError("Unrecognized algorithm for ALS!")
    optimizer.initialize_ground_truth_for_als()

    initial_fit = optimizer.compute_exact_fit()
    print(f"Initial Fit: {initial_fit}")
    optimizer.execute_ALS_rounds(args.iter, sample_count, args.epoch_iter)
    optimizer_stats = json.loads(optimizer.get_statistics_json())
    final_fit = optimizer.compute_exact_fit()

    output_dict = {
        "time": datetime.now().strftime("%m/%d/%Y, %H:%M:%S"),
        "metadata": args.metadata,
        "input": args.input,
        "target_rank": args.trank,
        "iterations": args.iter,
        "algorithm": args.algorithm,
        "preprocessing": args.preprocessing,
        "data_distribution": args.distribution,
        "sample_count": args.samples,
        "accuracy_epoch_length": args.epoch_iter,
        "trial_count": args.repetitions,
        "trial_num": trial_num,
        "initial_fit": initial_fit,
        "final_fit": final_fit,
        "thread_count": os.environ.get("OMP_NUM_THREADS"),
        "node_count": os.environ.get("NODE_COUNT"),
        "mpi_rank_count": 1,
        "precision": args.precision,
        "stats": optimizer_stats,
    }
    print(json.dumps(output_dict, indent=4))
    print(f"Final Fit: {final_fit}")
    if args.factor_file is not None:
        print(f"Factors written to {low_rank_tensor.write_to_file(args.factor_file)}")
    if output_filename is not None:
        with open(os.path.join(args.output_folder, output_filename), "w") as f:
            f.write(json.dumps(output_dict, indent=4))
    optimizer.deinitialize()
    return output_dict


def parse_args(argv=None):
    parser = argparse.ArgumentParser()
    parser.add_argument("-i", "--input", type=str, help="Tensor name to decompose", required=True)
    parser.add_argument("-t", "--trank", help="Rank of the target decomposition", required=True, type=int)
    parser.add_argument("-iter", help="Number of ALS iterations", required=True, type=int)
    parser.add_argument("-dist", "--distribution", type=str,
                        help="Data distribution (tensor_stationary / accumulator_stationary)", required=False)
    parser.add_argument("-alg", "--algorithm", type=str, help="Algorithm to perform decomposition")
    parser.add_argument("-s", "--samples", help="Number of samples taken from the KRP", required=False, type=int)
    parser.add_argument("-o", "--output_folder", help="Folder name to print statistics", required=False)
    parser.add_argument("-e", "--epoch_iter", help="Number of iterations per accuracy evaluation epoch",
                        required=False, type=int, default=5)
    parser.add_argument("-r", "--repetitions", help="Number of repetitions for multiple trials", required=False,
                        type=int, default=1)
    parser.add_argument("-m", "--metadata", help="A string piece of metadata to include output json",
                        required=False, type=str, default="")
    parser.add_argument("-p", "--preprocessing", help="Preprocessing algorithm to apply before randomized algorithms",
                        required=False, type=str)
    parser.add_argument("--seed", type=int, default=0, help="seed of the factor init and the sampling stream")
    parser.add_argument("--precision", default="fp64", choices=["fp64", "tf32", "bf16"])
    parser.add_argument("--factor-file", dest="factor_file", default=None,
                        help="write the factors (FACTOR_MODE_i, SIGMA) here at the end (HDF5 with h5py, else .npz)")
    parser.add_argument("--init-factors", dest="init_factors", default=None,
                        help="start from the factors of a --factor-file (resume)")
    return parser.parse_args(argv)


def remaining_trial(args):
    """Trial resume (decompose.py:188-214): the first trial number whose output
    file does not exist yet, or None when all are done."""
    if args.output_folder is None:
        return 0, None
    prefix = "_".join([args.input.replace(":", "-"), str(args.trank), str(args.iter), str(args.distribution),
                       str(args.algorithm), str(args.samples), str(args.epoch_iter)])
    if args.metadata is not None:
        prefix += f"_{args.metadata}"
    done = []
    for f in os.listdir(args.output_folder):
        if prefix in f:
            with open(os.path.join(args.output_folder, f)) as h:
                done.append(json.load(h)["trial_num"])
    left = [i for i in range(args.repetitions) if i not in done]
    if not left:
        return None, None
    return left[0], f"{prefix}_{left[0]}.out"


if __name__ == "__main__":
    a = parse_args()
    trial, fname = remaining_trial(a)
    if trial is None:
        print("No trials left to perform!")
    else:
        decompose(a, fname, trial)
