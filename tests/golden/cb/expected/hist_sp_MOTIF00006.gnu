set output "hist_sp_MOTIF00006.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-43.4339:17.4488]
set yrange [0:7246]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00006.dat" using 1:2 title 'MOTIF00006 (sp)' with boxes
