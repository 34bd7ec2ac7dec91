function [history_output, field_output, force_output, field_output_time] = fn_explicit_dynamic_solver_v5_gb300(...
    K, C, M, time, ...
    forcing_indices, forcing_functions, ...
    disp_indices, disp_functions, ...
    history_indices, field_output_every_n_frames, varargin)
%SUMMARY
%   Drop-in for fn_explicit_dynamic_solver_v5 on one GB300 GPU: the same 11
%   arguments and 4 outputs (code/internal/fn_explicit_dynamic_solver_v5.m:1-5),
%   with prescribed displacements and the reaction forces at them. The time
%   loop runs in libbfe_gb300 through the MEX gateway bfe_mex_v5 (FP64, as
%   the reference's v5).

ndf = size(K, 1);
if ndf ~= size(K, 2)
    error('K must be square matrix');
end
if size(C, 1) ~= ndf || size(C, 2) ~= ndf
    error('C must be square matrix, same size as K');
end
if size(M, 1) ~= ndf || size(M, 2) ~= ndf
    error('M must be square matrix, same size as K');
end
if isempty(forcing_functions)
    forcing_functions = zeros(0, numel(time));
end
if isempty(disp_functions)
    disp_functions = zeros(0, numel(time));
end

[history_output, field_output, force_output, field_output_time] = bfe_mex_v5(K, C, M, time(:).', ...
    forcing_indices(:), forcing_functions, disp_indices(:), disp_functions, history_indices(:), ...
    field_output_every_n_frames);

if isempty(history_indices)
    history_output = [];
end
if isempty(disp_indices)
    force_output = [];
end
if isinf(field_output_every_n_frames)
    field_output = [];
    field_output_time = [];
end
end
