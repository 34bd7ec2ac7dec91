function [history_output, field_output, force_output, field_output_time] = fn_explicit_dynamic_solver_gb300(...
    K, C, M, time, ...
    forcing_indices, forcing_functions, ...
    disp_indices, disp_functions, ...
    history_indices, field_output_every_n_frames, varargin)
%SUMMARY
%   Drop-in for fn_explicit_dynamic_solver_v6 on one GB300 GPU: the same 14
%   arguments and 4 outputs (code/internal/fn_explicit_dynamic_solver_v6.m:1-5),
%   plus an optional 15th, the builder's gl_lookup, which lets the FP32 plan
%   evaluate the stiffness product in its translation-invariant difference
%   form. The time loop runs in libbfe_gb300 through the MEX gateway bfe_mex.
%INPUTS (as v6)
%   varargin{1} use_gpu (the GPU is always used), varargin{2}
%   field_output_type (default 'KE'), varargin{3} solver_mode, varargin{4}
%   solver_precision ('double' or 'single'), varargin{5} gl_lookup
%OUTPUTS (as v6)
%   history_output - q x n, class of solver_precision ([] if no monitors)
%   field_output - ndf x n_frames, class of solver_precision ([] if none)
%   force_output - [] (prescribed displacements are an error, as v6's own
%   loop fails on them at v6.m:191)
%   field_output_time - 1 x n_frames

if numel(varargin) < 2
    field_output_type = 'KE';
else
    field_output_type = varargin{2};
end
if numel(varargin) < 3
    solver_mode = 'vel at current time step';   %v6's default spelling (v6.m:44), accepted by neither case
else
    solver_mode = varargin{3};
end
if numel(varargin) < 4
    solver_precision = 'double';
else
    solver_precision = varargin{4};
end
if numel(varargin) < 5
    gl_lookup = [];
else
    gl_lookup = varargin{5};
end

if size(K, 1) ~= size(K, 2)
    error('K must be square matrix');
end
if size(C, 1) ~= size(C, 2)
    error('C must be square matrix');
end
if size(M, 1) ~= size(M, 2)
    error('M must be square matrix');
end
if ~isempty(disp_indices)
    error('bfe:disp', 'prescribed displacements are not supported by the v6 path');
end
switch solver_mode
    case {'vel at last half time step', 'vel at curent time step'}
    otherwise
        error('bfe:mode', 'unknown solver_mode ''%s''', solver_mode);
end
switch field_output_type
    case {'mean(u1)', 'mean(u2)', 'mean(u3)', 'curl(u)', 'div(u)', 'raw(u)'}
        field_is_vel = 0;
    otherwise
        field_is_vel = 1;
end
if isempty(forcing_functions)
    forcing_functions = zeros(0, numel(time));
end

[history_output, field_output, field_output_time] = bfe_mex(K, C, M, time(:).', ...
    forcing_indices(:), forcing_functions, history_indices(:), field_output_every_n_frames, ...
    field_is_vel, solver_mode, solver_precision, gl_lookup);

if isempty(history_indices)
    history_output = [];
end
if isinf(field_output_every_n_frames)
    field_output = [];
    field_output_time = [];
end
force_output = [];
end
