"""GB300-native NCC template matching (mvkit FindNccModel / CreateNccModel)."""
from .ncc import (MvError, NccModel, DeviceImage, PinnedBuffer, create_ncc_model, deserialize_ncc_model,
                  find_ncc_model, find_ncc_model_stage, find_ncc_models, find_ncc_models_batch, get_ncc_model_params, load, ncc_refine_similarity, ncc_score_gradient, profile_enable, profile_read,
                  profile_reset, pyramid_level, read_ncc_model, serialize_ncc_model, set_correlation_path,
                  write_ncc_model, set_batch_merge, batch_profile_reset, batch_profile_read, set_budgets,
                  get_budgets, extended_budgets, ncc_quadratic_peak_fit)

__all__ = ["MvError", "NccModel", "DeviceImage", "PinnedBuffer", "create_ncc_model", "find_ncc_model",
           "find_ncc_model_stage", "find_ncc_models", "find_ncc_models_batch", "get_ncc_model_params", "load", "ncc_refine_similarity", "ncc_score_gradient", "profile_enable", "profile_read",
           "profile_reset", "pyramid_level", "set_correlation_path", "write_ncc_model", "read_ncc_model",
           "serialize_ncc_model", "deserialize_ncc_model", "set_batch_merge", "batch_profile_reset",
           "batch_profile_read", "set_budgets", "get_budgets", "extended_budgets",
           "ncc_quadratic_peak_fit"]
