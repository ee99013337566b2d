set output "hist_sp_MOTIF00007.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-68.0474:19.5363]
set yrange [0:8575]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00007.dat" using 1:2 title 'MOTIF00007 (sp)' with boxes
