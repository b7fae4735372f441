"""Test infrastructure: FP64 restatements of the f_number beamformer (the oracle).
Never imported by the product package."""
